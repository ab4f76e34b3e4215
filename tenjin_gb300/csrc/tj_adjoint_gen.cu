// Reverse mode of the FP64 update for the configurations the 2-D fluid
// adjoint (tj_adjoint.cu) does not cover: 1-, 2- and 3-D, solids with the
// 5-wave solver (hllc.cpp:133-380), the plastic radial return
// (plastic.cpp:83-223), cleanUpV, the radial source, every EOS -- one domain,
// MUSCL without BVD-THINC, no mixtures.
//
// The adjoint is accumulated from local Jacobians of the FP64 path's own
// device functions, evaluated in forward mode with the Dual instance
// (tj_dual.cuh): for each cell's update (update_cell, including the last
// direction's conservativeToPrimitive and the second stage's average,
// radial return, cleanUpV and cleanUpAlpha) and each face's Riemann problem
// (load_prim_face's closure and face_flux), one pass per input with that
// input's direction set gives one column of the local Jacobian, whose dot
// product with the output adjoint is that input's adjoint. The MUSCL
// reconstruction is linear on its active branch (the van Leer slope of this
// form is u0 - um or up - u0) and is reversed directly. Every reverse kernel
// gathers (a cell from its faces and stencil, a face from its two cells);
// nothing is summed with atomics, and the EOS-parameter adjoints are summed
// per parameter in a fixed order, so the gradient is deterministic.
//
// The update of every direction but the last of a stage is affine in the
// accumulator and the fluxes (bilinear in the non-conservative terms) and is
// reversed by hand.
//
// Cost: a local Jacobian takes as many passes as the operator has inputs
// (about 100 for a copper cell's last-direction update, 34 for a copper
// face), so a backward step costs tens of forward steps: the general reverse
// mode is exact and deterministic; the 2-D fluid adjoint is the fast one
// (backward about 3 forward steps).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "tj_dual.cuh"
#include "tj_dual_path.cuh"
#include "tj_path.cuh"
#include "tj_path_launch.cuh"
#include "tj_adjoint_gen.cuh"

namespace tj {

namespace {

constexpr int kGT = 128;  // threads per block of the reverse kernels
constexpr int kNS = 48;   // carried words (39 at most: 4 solid plastic materials)
constexpr int kNX = 32;   // flux words (29 at most)
constexpr int kNF = 32;   // face-state words (31 at most)

inline int gblocks(long long n)
{
    long long b = (n + kGT - 1) / kGT;
    return (int)std::max(1LL, std::min(b, 152LL * 32));
}

struct FacePairLocal {
    const Dual* F0;
    const Dual* F1;
    __device__ __forceinline__ Dual operator()(int w, int s) const { return s ? F1[w] : F0[w]; }
};

// One forward-mode pass of a cell's update: the output's tangent dotted with
// the output adjoint lo. Yw / Aw are work copies of the accumulator and U^n.
__device__ __noinline__ double upd_pass(const DevParamsT& P, const PathBufs<Dual>& lb, const Dual* X, const Dual* Y,
                                        const Dual* A, Dual* Yw, Dual* Aw, const Dual* F0, const Dual* F1,
                                        const double* lo, const DevDomain& D, int i, int d, int first, int last,
                                        int finish, Dual dtv)
{
    for (int w = 0; w < P.NS; ++w) {
        Yw[w] = Y[w];
        Aw[w] = A[w];
    }
    update_cell(P, lb, X, Yw, 0LL, D, i, d, first, last, finish, dtv, FacePairLocal{F0, F1});
    const Dual* out = finish ? Aw : Yw;
    double s = 0.0;
    for (int w = 0; w < P.NS; ++w)
        if (lo[w] != 0.0) s += lo[w] * out[w].d;  // a zero adjoint takes no part
    return s;
}

// ---------------------------------------------------------------------------
// Update of one direction, reversed per cell. Inputs: the accumulator Yin
// (not read by the first direction, whose accumulator is U), the stage input
// U, the two face fluxes F0 / F1 and, with the finish, U^n (A0). The output
// adjoint lamOut is that of the direction's output (the next accumulator, or
// U^{n+1} for the finish). Writes the adjoints of Yin and of the two fluxes
// (per cell: F0 of the face below, F1 of the face above), adds those of U and
// A0, and adds each EOS parameter's part into geos (per cell).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kGT) k_gen_upd_rev(DevParamsT P, Fp64Bufs fb, const double* Yin, const double* U,
                                                     const double* A0, const double* lamOut, double* lamYin,
                                                     double* lamU, double* lamA0, double* lamF0, double* lamF1,
                                                     double* geos, int d, int first, int last, int finish, int npar)
{
    const long long nt = fb.ntot, nf = fb.nftot[d];
    const int NS = P.NS, NX = P.NX;
    const DevDomain D = fb.doms[0];
    const Dual dtv(fb.scal->dt);
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        split3(g - D.off, D.n[0], D.n[1], i, j, k);
        int o[3] = {0, 0, 0};
        o[d] = 1;
        const long long f0 = face_index(D, d, i, j, k), f1 = face_index(D, d, i + o[0], j + o[1], k + o[2]);
        Dual X[kNS], Y[kNS], A[kNS], Yw[kNS], Aw[kNS], F0[kNX], F1[kNX];
        double lo[kNS];
        for (int w = 0; w < NS; ++w) {
            X[w] = Dual(U[w * nt + g]);
            Y[w] = Dual(first ? 0.0 : Yin[w * nt + g]);
            A[w] = Dual(finish ? A0[w * nt + g] : 0.0);
            lo[w] = lamOut[w * nt + g];
        }
        for (int w = 0; w < NX; ++w) {
            F0[w] = Dual(fb.FX[w * nf + f0]);
            F1[w] = Dual(fb.FX[w * nf + f1]);
        }
        int cb = fb.cell_box[g];
        PathBufs<Dual> lb{};
        lb.ntot = 1;
        lb.A = Aw;
        lb.cell_box = &cb;
        lb.scal = fb.scal;
#define TJ_PASS(PP) upd_pass(PP, lb, X, Y, A, Yw, Aw, F0, F1, lo, D, i, d, first, last, finish, dtv)
        if (!first)
            for (int w = 0; w < NS; ++w) {
                Y[w].d = 1.0;
                lamYin[w * nt + g] = TJ_PASS(P);
                Y[w].d = 0.0;
            }
        for (int w = 0; w < NS; ++w) {
            X[w].d = 1.0;
            lamU[w * nt + g] += TJ_PASS(P);
            X[w].d = 0.0;
        }
        for (int w = 0; w < NX; ++w) {
            F0[w].d = 1.0;
            lamF0[w * nt + g] = TJ_PASS(P);
            F0[w].d = 0.0;
            F1[w].d = 1.0;
            lamF1[w * nt + g] = TJ_PASS(P);
            F1[w].d = 0.0;
        }
        if (finish)
            for (int w = 0; w < NS; ++w) {
                A[w].d = 1.0;
                lamA0[w * nt + g] += TJ_PASS(P);
                A[w].d = 0.0;
            }
        if (geos && npar > 0) {
            DevParamsT Q = P;
            for (int m = 0; m < P.M; ++m)
                for (int q = 0; q < npar; ++q) {
                    Q.prm[m][q].d = 1.0;
                    geos[(long long)(m * npar + q) * nt + g] += TJ_PASS(Q);
                    Q.prm[m][q].d = 0.0;
                }
        }
#undef TJ_PASS
    }
}

// ---------------------------------------------------------------------------
// Update of a direction other than the last, reversed per cell by hand: it
// only adds dt/dx times flux differences to the conserved words, with the
// non-conservative terms -alpha (S*_0 - S*_1) and -(2/3) V (S*_0 - S*_1) +
// u_row (V*_0 - V*_1) (hllc.cpp:493-523), so the accumulator's adjoint passes
// through and the flux and stage-input adjoints are its products with dt/dx
// and those terms' factors.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kGT) k_gen_upd_rev_lin(DevParams P, Fp64Bufs fb, const double* U,
                                                         const double* lamOut, double* lamYin, double* lamU,
                                                         double* lamF0, double* lamF1, int d, int first)
{
    const long long nt = fb.ntot, nf = fb.nftot[d];
    const int NS = P.NS, NX = P.NX;
    const DevDomain D = fb.doms[0];
    const double dtdx = fb.scal->dt / D.dx[d];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        split3(g - D.off, D.n[0], D.n[1], i, j, k);
        int o[3] = {0, 0, 0};
        o[d] = 1;
        const long long f0 = face_index(D, d, i, j, k), f1 = face_index(D, d, i + o[0], j + o[1], k + o[2]);
        double l0[kNX], l1[kNX];
        for (int w = 0; w < NX; ++w) l0[w] = l1[w] = 0.0;
        auto lo = [&](int w) { return lamOut[(long long)w * nt + g]; };
        auto u = [&](int w) { return U[(long long)w * nt + g]; };
        const double dS = fb.FX[(long long)P.X_SSTAR * nf + f0] - fb.FX[(long long)P.X_SSTAR * nf + f1];
        double su = 0.0;  // adjoint of S*_0 - S*_1
        for (int m = 0; m < P.M; ++m) {
            const double la = lo(P.S_ALPHA + m);
            l0[P.X_ALPHA + m] += dtdx * la;
            l1[P.X_ALPHA + m] -= dtdx * la;
            su -= dtdx * u(P.S_ALPHA + m) * la;
            lamU[(long long)(P.S_ALPHA + m) * nt + g] -= dtdx * dS * la;
            const double lr = lo(P.S_ARHO + m);
            l0[P.X_ARHO + m] += dtdx * lr;
            l1[P.X_ARHO + m] -= dtdx * lr;
            if (P.plastic) {
                const double le = lo(P.S_ARE + m);
                l0[P.X_ARE + m] += dtdx * le;
                l1[P.X_ARE + m] -= dtdx * le;
            }
        }
        for (int r = 0; r < 3; ++r) {
            const double lm = lo(P.S_RHOU + r);
            l0[P.X_RHOU + r] += dtdx * lm;
            l1[P.X_RHOU + r] -= dtdx * lm;
        }
        l0[P.X_E] += dtdx * lo(P.S_E);
        l1[P.X_E] -= dtdx * lo(P.S_E);
        if (P.solid)
            for (int qq = 0; qq < 9; ++qq) {
                const int row = qq / 3, col = qq % 3;
                const double lv = lo(P.S_V + qq);
                l0[P.X_V + qq] += dtdx * lv;
                l1[P.X_V + qq] -= dtdx * lv;
                su -= dtdx * (2.0 / 3.0) * u(P.S_V + qq) * lv;
                lamU[(long long)(P.S_V + qq) * nt + g] -= dtdx * (2.0 / 3.0) * dS * lv;
                const double dV = fb.FX[(long long)(P.X_VSTAR + col) * nf + f0] - fb.FX[(long long)(P.X_VSTAR + col) * nf + f1];
                l0[P.X_VSTAR + col] += dtdx * u(P.S_VEL + row) * lv;
                l1[P.X_VSTAR + col] -= dtdx * u(P.S_VEL + row) * lv;
                lamU[(long long)(P.S_VEL + row) * nt + g] += dtdx * dV * lv;
            }
        l0[P.X_SSTAR] += su;
        l1[P.X_SSTAR] -= su;
        for (int w = 0; w < NX; ++w) {
            lamF0[(long long)w * nt + g] = l0[w];
            lamF1[(long long)w * nt + g] = l1[w];
        }
        // the accumulator passes through: to U for the first direction
        for (int w = 0; w < NS; ++w) {
            if (first) lamU[(long long)w * nt + g] += lo(w);
            else lamYin[(long long)w * nt + g] = lo(w);
        }
    }
}

// One forward-mode pass of a face's Riemann problem from its two stored
// states: the flux's tangent dotted with the flux adjoint lF.
__device__ __noinline__ double flux_pass(const DevParamsT& P, const Dual* Lp, const Dual* Rp, Dual* Fo, const double* lF,
                                         int oddl, int oddr, int d, DevScalars* scal)
{
    CellT<Dual> L, R;
    load_prim_face(P, Lp, 1LL, 0LL, oddl, L);
    load_prim_face(P, Rp, 1LL, 0LL, oddr, R);
    FluxV<Dual> F;
    Dual Ss, vstar[3] = {Dual(0.0), Dual(0.0), Dual(0.0)};
    face_flux(P, L, R, d, F, Ss, vstar, scal);
    for (int w = 0; w < P.NX; ++w) Fo[w] = Dual(0.0);
    store_flux(P, Fo, 1LL, 0LL, F, Ss, vstar);
    double s = 0.0;
    for (int w = 0; w < P.NX; ++w)
        if (lF[w] != 0.0) s += lF[w] * Fo[w].d;
    return s;
}

// ---------------------------------------------------------------------------
// Riemann problem of one face, reversed: the face's flux adjoint is gathered
// from the cell above (its F0) and the cell below (its F1); one pass per
// word of the two stored face states (UR of the cell below, UL of the cell
// above, boundary images as k_flux maps them) gives their adjoints, per face.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kGT) k_gen_flux_rev(DevParamsT P, Fp64Bufs fb, const double* lamF0,
                                                      const double* lamF1, double* lamLf, double* lamRf,
                                                      double* geos_f, int d, int npar, int nfw)
{
    const long long nt = fb.ntot, nf = fb.nftot[d];
    const int NX = P.NX;
    const DevDomain D = fb.doms[0];
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x) {
        int nfv[3] = {D.n[0], D.n[1], D.n[2]};
        nfv[d] += 1;
        int i, j, k;
        split3(f - D.foff[d], nfv[0], nfv[1], i, j, k);
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int idx[3] = {i, j, k};
        int rl[3], rr[3];
        const long long gl = map_cell(P, D, i - o[0], j - o[1], k - o[2], rl);
        const long long gr = map_cell(P, D, i, j, k, rr);
        double lF[kNX];
        for (int w = 0; w < NX; ++w) {
            double s = 0.0;
            if (idx[d] >= 1) s += lamF1[w * nt + D.off + (i - o[0]) + (long long)D.n[0] * ((j - o[1]) + (long long)D.n[1] * (k - o[2]))];
            if (idx[d] < D.n[d]) s += lamF0[w * nt + D.off + i + (long long)D.n[0] * (j + (long long)D.n[1] * k)];
            lF[w] = s;
        }
        Dual Lp[kNF], Rp[kNF], Fo[kNX];
        for (int w = 0; w < nfw; ++w) {
            Lp[w] = Dual(fb.UR[w * nt + gl]);
            Rp[w] = Dual(fb.UL[w * nt + gr]);
        }
#define TJ_PASS(PP) flux_pass(PP, Lp, Rp, Fo, lF, rl[d] ? d : -1, rr[d] ? d : -1, d, fb.scal)
        for (int w = 0; w < nfw; ++w) {
            Lp[w].d = 1.0;
            lamLf[w * nf + f] = TJ_PASS(P);
            Lp[w].d = 0.0;
            Rp[w].d = 1.0;
            lamRf[w * nf + f] = TJ_PASS(P);
            Rp[w].d = 0.0;
        }
        if (geos_f && npar > 0) {
            DevParamsT Q = P;
            for (int m = 0; m < P.M; ++m)
                for (int q = 0; q < npar; ++q) {
                    Q.prm[m][q].d = 1.0;
                    geos_f[(long long)(m * npar + q) * nf + f] += TJ_PASS(Q);
                    Q.prm[m][q].d = 0.0;
                }
        }
#undef TJ_PASS
    }
}

// The carried word a face-state word (store_prim_face) is made of, and
// whether MUSCL reconstructs it (otherwise it is the cell's own value).
__device__ __forceinline__ int face_src(const DevParams& P, int w, bool& rec)
{
    rec = true;
    if (w < P.M) return P.S_ALPHA + w;
    w -= P.M;
    if (w < P.M) return P.S_RHOK + w;
    w -= P.M;
    if (w < 3) return P.S_VEL + w;
    w -= 3;
    if (w == 0) return P.S_P;
    w -= 1;
    if (P.solid) {
        if (w < 9) return P.S_V + w;
        w -= 9;
        if (!P.any_solid) {
            if (w == 0) {
                rec = false;
                return P.S_HJ2;
            }
            w -= 1;
        }
    }
    // plastic: epsilon of a solid (reconstructed), alphaRhoEps of a fluid (copied)
    if (P.phase[w] == TJ_PHASE_SOLID) return P.S_EPS + w;
    rec = false;
    return P.S_ARE + w;
}

// ---------------------------------------------------------------------------
// MUSCL reconstruction, reversed per cell h: the adjoints of UL / UR of the
// cells whose stencil holds h (h - 1, h, h + 1 along d, boundary images
// included) times the active branch's coefficients, added to h's carried
// words of the stage input.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kGT) k_gen_recon_rev(DevParams P, Fp64Bufs fb, const double* X,
                                                       const double* lamLf, const double* lamRf, double* lamU, int d,
                                                       int nfw)
{
    const long long nt = fb.ntot, nf = fb.nftot[d];
    const DevDomain D = fb.doms[0];
    for (long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x; h < nt; h += (long long)gridDim.x * blockDim.x) {
        int c[3];
        split3(h - D.off, D.n[0], D.n[1], c[0], c[1], c[2]);
        const int n = D.n[d];
        double acc[kNF];
        for (int w = 0; w < nfw; ++w) acc[w] = 0.0;
        for (int kq = -1; kq <= 1; ++kq) {
            int kc[3] = {c[0], c[1], c[2]};
            kc[d] += kq;
            if (kc[d] < 0 || kc[d] >= n) continue;
            // adjoints of UL / UR of cell kc (faces below and above, and the
            // boundary face whose ghost side is this cell's state)
            int lo[3] = {kc[0], kc[1], kc[2]}, hi[3] = {kc[0], kc[1], kc[2]};
            hi[d] += 1;
            const long long fl = face_index(D, d, lo[0], lo[1], lo[2]), fh = face_index(D, d, hi[0], hi[1], hi[2]);
            int e0[3] = {kc[0], kc[1], kc[2]}, en[3] = {kc[0], kc[1], kc[2]};
            e0[d] = 0;
            en[d] = n;
            const long long fz = face_index(D, d, e0[0], e0[1], e0[2]), fn = face_index(D, d, en[0], en[1], en[2]);
            // the stencil of kc, mapped
            int rf[3][3];
            long long gs[3];
            for (int q = 0; q < 3; ++q) {
                int s[3] = {kc[0], kc[1], kc[2]};
                s[d] += q - 1;
                gs[q] = map_cell(P, D, s[0], s[1], s[2], rf[q]);
            }
            for (int w = 0; w < nfw; ++w) {
                const double lR = lamLf[w * nf + fh] + (kc[d] == 0 ? lamLf[w * nf + fz] : 0.0);
                const double lL = lamRf[w * nf + fl] + (kc[d] == n - 1 ? lamRf[w * nf + fn] : 0.0);
                bool rec;
                const int src = face_src(P, w, rec);
                if (!rec || !P.muscl) {
                    if (gs[1] == h) acc[w] += lL + lR;
                    continue;
                }
                const bool vd = (src == P.S_VEL + d);
                double u[3];
                for (int q = 0; q < 3; ++q) {
                    const double v = X[src * nt + gs[q]];
                    u[q] = (vd && rf[q][d]) ? -v : v;
                }
                double rr = (u[1] - u[0]) / (u[2] - u[1]);
                if (isinf(rr) || isnan(rr)) rr = 0.0;
                double b1 = 0.0, b2 = 0.0;
                if (rr > 0.0) {
                    const double a = 2.0 / (1.0 + rr), b = 2.0 * rr / (1.0 + rr);
                    if (b < a) b1 = 1.0;
                    else b2 = 1.0;
                }
                // L = u0 - g / 2, R = u0 + g / 2 with g = b1 (u0 - um) + b2 (up - u0)
                const double cL[3] = {0.5 * b1, 1.0 - 0.5 * (b1 - b2), -0.5 * b2};
                const double cR[3] = {-0.5 * b1, 1.0 + 0.5 * (b1 - b2), 0.5 * b2};
                for (int q = 0; q < 3; ++q)
                    if (gs[q] == h) {
                        const double sg = (vd && rf[q][d]) ? -1.0 : 1.0;
                        acc[w] += sg * (cL[q] * lL + cR[q] * lR);
                    }
            }
        }
        for (int w = 0; w < nfw; ++w) {
            bool rec;
            const int src = face_src(P, w, rec);
            lamU[src * nt + h] += acc[w];
        }
    }
}

// One forward-mode pass of the initial closure of one cell.
__device__ __noinline__ double p2c_pass(const DevParamsT& P, const Dual* pr, Dual* out, const double* lo)
{
    CellT<Dual> c;
    int w = 0;
    for (int m = 0; m < P.M; ++m) c.alpha[m] = pr[w++];
    for (int m = 0; m < P.M; ++m) c.rhok[m] = pr[w++];
    for (int r = 0; r < 3; ++r) c.vel[r] = pr[w++];
    c.p = pr[w++];
    c.hj2 = Dual(0.0);
    if (P.solid)
        for (int q = 0; q < 9; ++q) c.V[q] = pr[w++];
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) c.eps[m] = pr[w++];
    p2c(P, c);
    store_state(P, out, 1LL, 0LL, c);
    double s = 0.0;
    for (int q = 0; q < P.NS; ++q)
        if (lo[q] != 0.0) s += lo[q] * out[q].d;
    return s;
}

// primitiveToConservative of the initial state, reversed per cell: the
// adjoints of the primitives (tj_set_primitive layout) and each EOS
// parameter's part.
__global__ void __launch_bounds__(kGT) k_gen_p2c_rev(DevParamsT P, Fp64Bufs fb, const double* prim,
                                                     const double* lamA, double* gprim, double* geos, int npar,
                                                     int nprim)
{
    const long long nt = fb.ntot;
    const int NS = P.NS;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt; t += (long long)gridDim.x * blockDim.x) {
        Dual pr[kNF], out[kNS];
        double lo[kNS];
        for (int w = 0; w < nprim; ++w) pr[w] = Dual(prim[w * nt + t]);
        for (int w = 0; w < NS; ++w) lo[w] = lamA[w * nt + t];
        for (int w = 0; w < nprim; ++w) {
            pr[w].d = 1.0;
            gprim[w * nt + t] = p2c_pass(P, pr, out, lo);
            pr[w].d = 0.0;
        }
        if (geos && npar > 0) {
            DevParamsT Q = P;
            for (int m = 0; m < P.M; ++m)
                for (int q = 0; q < npar; ++q) {
                    Q.prm[m][q].d = 1.0;
                    geos[(long long)(m * npar + q) * nt + t] += p2c_pass(Q, pr, out, lo);
                    Q.prm[m][q].d = 0.0;
                }
        }
    }
}

// Sum of n entries per parameter, in a fixed order (one block per parameter,
// a fixed stride per thread, a fixed tree): out[p] += sum_e v[p * n + e].
__global__ void k_gen_sum(const double* v, long long n, double* out)
{
    __shared__ double s[256];
    const int p = blockIdx.x;
    double a = 0.0;
    for (long long e = threadIdx.x; e < n; e += 256) a += v[(long long)p * n + e];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[p] += s[0];
}

// AccessPattern gradient -> carried-word adjoint (derived components dropped).
__global__ void k_gen_ap_to_lam(const double* ap, const int* a_to_s, int ncomp, long long nt, double* lam, int ns)
{
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt; t += (long long)gridDim.x * blockDim.x) {
        for (int w = 0; w < ns; ++w) lam[w * nt + t] = 0.0;
        for (int a = 0; a < ncomp; ++a)
            if (a_to_s[a] >= 0) lam[a_to_s[a] * nt + t] = ap[a * nt + t];
    }
}

DevParamsT params_t(const DevParams& D)
{
    DevParamsT P;
    std::memset(&P, 0, sizeof P);
    P.dim = D.dim; P.M = D.M; P.solid = D.solid; P.thinc = D.thinc; P.plastic = D.plastic; P.muscl = D.muscl;
    P.any_solid = D.any_solid; P.radial = D.radial; P.nmix = D.nmix; P.reactive = D.reactive;
    for (int d = 0; d < 3; ++d) {
        P.lo_bc[d] = D.lo_bc[d];
        P.hi_bc[d] = D.hi_bc[d];
    }
    P.cfl = Dual(D.cfl);
    P.beta = Dual(D.beta);
    for (int m = 0; m < TJ_MAX_MAT; ++m) {
        P.phase[m] = D.phase[m];
        P.eos[m] = D.eos[m];
        P.yield[m] = Dual(D.yield[m]);
        for (int k = 0; k < TJ_MAX_EOS_PARAMS; ++k) P.prm[m][k] = Dual(D.prm[m][k]);
    }
#define CP(f) P.f = D.f
    CP(S_ALPHA); CP(S_ARHO); CP(S_RHOK); CP(S_RHO); CP(S_RHOU); CP(S_VEL); CP(S_E); CP(S_P); CP(S_V); CP(S_HJ2);
    CP(S_EPS); CP(S_ARE); CP(NS); CP(S_RMIX); CP(S_LAM); CP(S_ARL);
    CP(F_ALPHA); CP(F_ARHO); CP(F_RHO); CP(F_RHOU); CP(F_VEL); CP(F_E); CP(F_P); CP(F_A); CP(F_SIGMA); CP(F_V);
    CP(F_ARE); CP(NF); CP(F_ARL);
    CP(X_ALPHA); CP(X_ARHO); CP(X_RHOU); CP(X_E); CP(X_SSTAR); CP(X_V); CP(X_VSTAR); CP(X_ARE); CP(NX); CP(X_ARL);
#undef CP
    P.S_ELO = -1;
    return P;
}

}  // namespace

struct GenAdj {
    int nsteps = 0, stride = 0, nck = 0, npar = 0, nprim = 0;
    long long N = 0;
    std::vector<double> dt;
    std::vector<double*> bufs;
    double *ck = nullptr, *ring = nullptr, *yout = nullptr, *acopy = nullptr, *yscr = nullptr, *yscr2 = nullptr;
    double *lamA = nullptr, *lamB = nullptr, *lamU = nullptr, *lamY0 = nullptr, *lamY1 = nullptr;
    double *lamF0 = nullptr, *lamF1 = nullptr, *lamLf = nullptr, *lamRf = nullptr, *geos = nullptr, *geosf = nullptr;
    double *prim0 = nullptr, *gsum = nullptr;
    int* a_to_s = nullptr;
    long long made[8] = {};  // the sizes the buffers were made for (gen_alloc)
};

GenAdj* gen_create() { return new GenAdj(); }

static void gen_free(GenAdj* a)
{
    for (double* p : a->bufs)
        if (p) cudaFree(p);
    a->bufs.clear();
    if (a->a_to_s) cudaFree(a->a_to_s);
    a->a_to_s = nullptr;
    for (long long& m : a->made) m = 0;
}

void gen_destroy(GenAdj* a)
{
    if (!a) return;
    gen_free(a);
    delete a;
}

const char* gen_unsupported(const DevParams& P, int ndom)
{
    if (ndom != 1) return "the adjoint covers one domain";
    const int nfw = 2 * P.M + 4 + (P.solid ? 9 + (P.any_solid ? 0 : 1) : 0) + (P.plastic ? P.M : 0);
    if (P.NS > kNS || P.NX > kNX || nfw > kNF || P.NCOMP > 64)
        return "the general adjoint's per-cell arrays are smaller than this layout";
    if (P.thinc) return "the general adjoint covers MUSCL without BVD-THINC (2-D fluids with THINC: the 2-D adjoint)";
    if (P.nmix) return "the adjoint covers no mixtures";
    return nullptr;
}

static int gen_alloc(GenAdj* a, const DevParams& P, const Fp64Bufs& b, int nsteps, int stride)
{
    const long long N = b.ntot;
    const int nck = (nsteps + stride - 1) / stride;
    const long long nfmax = std::max(b.nftot[0], std::max(b.nftot[1], b.nftot[2]));
    const long long want[8] = {N, nck, stride, P.NS, P.NX, P.NF, nfmax, (long long)P.M * 16 + P.dim};
    bool same = true;
    for (int k = 0; k < 8; ++k) same &= a->made[k] == want[k];
    if (same) return TJ_OK;
    gen_free(a);
    auto al = [&](double** p, size_t n) {
        if (cudaMalloc(p, sizeof(double) * std::max<size_t>(n, 1)) != cudaSuccess) return false;
        a->bufs.push_back(*p);
        return true;
    };
    const size_t S = (size_t)P.NS * N;
    const int mp = P.M * TJ_MAX_EOS_PARAMS;
    bool ok = al(&a->ck, S * nck) && al(&a->ring, S * stride) && al(&a->yout, S * 2 * P.dim) && al(&a->acopy, S) &&
              al(&a->yscr, S) && al(&a->yscr2, S) && al(&a->lamA, S) && al(&a->lamB, S) && al(&a->lamU, S) &&
              al(&a->lamY0, S) && al(&a->lamY1, S) && al(&a->lamF0, (size_t)P.NX * N) &&
              al(&a->lamF1, (size_t)P.NX * N) && al(&a->lamLf, (size_t)P.NF * nfmax) &&
              al(&a->lamRf, (size_t)P.NF * nfmax) && al(&a->geos, (size_t)mp * N) &&
              al(&a->geosf, (size_t)mp * nfmax) && al(&a->prim0, (size_t)P.NS * N) && al(&a->gsum, mp);
    ok = ok && cudaMalloc(&a->a_to_s, sizeof(int) * 64) == cudaSuccess;
    if (!ok) {
        gen_free(a);
        return TJ_ERR_CUDA;
    }
    for (int k = 0; k < 8; ++k) a->made[k] = want[k];
    return TJ_OK;
}

long long gen_forward(GenAdj* a, const DevParams& P, const Fp64Bufs& b, const double* prim, int nprim, const double* dt,
                      int nsteps, int stride, cudaStream_t st)
{
    if (nsteps < 1 || stride < 1) return TJ_ERR_ARG;
    stride = std::min(stride, nsteps);
    int e = gen_alloc(a, P, b, nsteps, stride);
    if (e) return e;
    a->nsteps = nsteps;
    a->stride = stride;
    a->nck = (nsteps + stride - 1) / stride;
    a->N = b.ntot;
    a->nprim = nprim;
    a->dt.assign(dt, dt + nsteps);
    cudaMemcpyAsync(a->prim0, prim, sizeof(double) * nprim * b.ntot, cudaMemcpyDeviceToDevice, st);
    const size_t S = (size_t)P.NS * b.ntot;
    long long launches = 0;
    for (int n = 0; n < nsteps; ++n) {
        if (n % stride == 0) cudaMemcpyAsync(a->ck + (size_t)(n / stride) * S, b.A, sizeof(double) * S, cudaMemcpyDeviceToDevice, st);
        launches += fp64_set_dt(b, dt[n], st);
        launches += fp64_stage(P, b, b.A, b.B, 0, st);
        launches += fp64_stage(P, b, b.B, b.C, 1, st);
    }
    return launches;
}

long long gen_backward(GenAdj* a, const DevParams& P, const Fp64Bufs& b, const double* grad_ap, double* grad_prim,
                       double* grad_eos, const int* nparams, cudaStream_t st)
{
    if (!a || a->nck == 0 || a->N != b.ntot) return TJ_ERR_STATE;
    const long long N = b.ntot;
    const size_t S = (size_t)P.NS * N;
    const DevParamsT PT = params_t(P);
    const int dim = P.dim;
    const int nfw = 2 * P.M + 4 + (P.solid ? 9 + (P.any_solid ? 0 : 1) : 0) + (P.plastic ? P.M : 0);
    int npar = 0;
    for (int m = 0; m < P.M; ++m) npar = std::max(npar, std::min(nparams[m], TJ_MAX_EOS_PARAMS));
    const int mp = P.M * npar;
    long long launches = 0;
    // the final adjoint in the carried layout
    int a2s[64];
    for (int k = 0; k < 64; ++k) a2s[k] = -1;
    auto map = [&](int a0, int s0, int n) {
        if (a0 >= 0 && s0 >= 0)
            for (int k = 0; k < n; ++k) a2s[a0 + k] = s0 + k;
    };
    map(P.A_ALPHA, P.S_ALPHA, P.M);
    map(P.A_ARHO, P.S_ARHO, P.M);
    map(P.A_RHOK, P.S_RHOK, P.M);
    map(P.A_RHO, P.S_RHO, 1);
    map(P.A_RHOU, P.S_RHOU, 3);
    map(P.A_VEL, P.S_VEL, 3);
    map(P.A_E, P.S_E, 1);
    map(P.A_P, P.S_P, 1);
    if (P.solid) {
        map(P.A_V, P.S_V, 9);
        map(P.A_HJ2, P.S_HJ2, 1);
    }
    if (P.plastic) {
        map(P.A_EPS, P.S_EPS, P.M);
        map(P.A_ARE, P.S_ARE, P.M);
    }
    cudaMemcpyAsync(a->a_to_s, a2s, sizeof(int) * P.NCOMP, cudaMemcpyHostToDevice, st);
    k_gen_ap_to_lam<<<gblocks(N), kGT, 0, st>>>(grad_ap, a->a_to_s, P.NCOMP, N, a->lamA, P.NS);
    ++launches;
    cudaMemsetAsync(a->geos, 0, sizeof(double) * std::max(mp, 1) * N, st);
    cudaMemsetAsync(a->gsum, 0, sizeof(double) * std::max(mp, 1), st);

    Fp64Bufs fb = b;
    fb.rec = nullptr;
    fb.rec_code = nullptr;
    double* Yout[2][3];
    for (int s = 0; s < 2; ++s)
        for (int d = 0; d < 3; ++d) Yout[s][d] = d < dim ? a->yout + (size_t)(s * dim + d) * S : nullptr;
    // EOS parts of the faces: summed per direction after each flux reversal
    auto fold_faces = [&](int d) {
        if (mp > 0) {
            k_gen_sum<<<mp, 256, 0, st>>>(a->geosf, b.nftot[d], a->gsum);
            ++launches;
        }
    };
    // one direction of one stage, reversed; lamOut -> lamYin; adds into lamU
    // (stage input) and lamA0 (U^n, the finish)
    auto rev_dir = [&](const double* U, const double* Yin, const double* A0, const double* lamOut, double* lamYin,
                       double* lamU, double* lamA0, int d, int first, int last, int finish) {
        // the forward reconstruction and fluxes of this direction
        Fp64Bufs f2 = fb;
        launches += path_dir_any(P, f2, U, a->yscr2, d, 1, 0, 0, st, nullptr);
        if (mp > 0) cudaMemsetAsync(a->geosf, 0, sizeof(double) * mp * b.nftot[d], st);
        if (!last && !finish)
            k_gen_upd_rev_lin<<<gblocks(N), kGT, 0, st>>>(P, fb, U, lamOut, lamYin, lamU, a->lamF0, a->lamF1, d, first);
        else
            k_gen_upd_rev<<<gblocks(N), kGT, 0, st>>>(PT, fb, Yin, U, A0, lamOut, lamYin, lamU, lamA0, a->lamF0,
                                                      a->lamF1, mp > 0 ? a->geos : nullptr, d, first, last, finish, npar);
        k_gen_flux_rev<<<gblocks(b.nftot[d]), kGT, 0, st>>>(PT, fb, a->lamF0, a->lamF1, a->lamLf, a->lamRf,
                                                            mp > 0 ? a->geosf : nullptr, d, npar, nfw);
        k_gen_recon_rev<<<gblocks(N), kGT, 0, st>>>(P, fb, U, a->lamLf, a->lamRf, lamU, d, nfw);
        launches += 3;
        fold_faces(d);
    };

    for (int ci = a->nck - 1; ci >= 0; --ci) {
        const int n0 = ci * a->stride, n1 = std::min(a->nsteps, n0 + a->stride);
        // recompute the interval's step inputs
        Fp64Bufs fr = fb;
        fr.A = a->acopy;
        cudaMemcpyAsync(a->acopy, a->ck + (size_t)ci * S, sizeof(double) * S, cudaMemcpyDeviceToDevice, st);
        for (int n = n0; n < n1; ++n) {
            cudaMemcpyAsync(a->ring + (size_t)(n - n0) * S, a->acopy, sizeof(double) * S, cudaMemcpyDeviceToDevice, st);
            if (n + 1 == n1) break;
            launches += fp64_set_dt(fr, a->dt[n], st);
            launches += fp64_stage(P, fr, a->acopy, a->yscr, 0, st);
            launches += fp64_stage(P, fr, a->yscr, a->yscr2, 1, st);
        }
        for (int n = n1 - 1; n >= n0; --n) {
            const double* An = a->ring + (size_t)(n - n0) * S;
            launches += fp64_set_dt(fb, a->dt[n], st);
            // stage intermediates: the output of every direction
            for (int d = 0; d < dim; ++d) {
                launches += path_dir_any(P, fb, An, a->yscr, d, d == 0, d == dim - 1, 0, st, nullptr);
                cudaMemcpyAsync(Yout[0][d], a->yscr, sizeof(double) * S, cudaMemcpyDeviceToDevice, st);
            }
            const double* B = Yout[0][dim - 1];
            Fp64Bufs f3 = fb;
            f3.A = a->acopy;
            cudaMemcpyAsync(a->acopy, An, sizeof(double) * S, cudaMemcpyDeviceToDevice, st);
            for (int d = 0; d < dim - 1; ++d) {
                launches += path_dir_any(P, f3, B, a->yscr, d, d == 0, 0, 0, st, nullptr);
                cudaMemcpyAsync(Yout[1][d], a->yscr, sizeof(double) * S, cudaMemcpyDeviceToDevice, st);
            }
            // stage 2 reversed: lamA is the adjoint of U^{n+1}
            cudaMemsetAsync(a->lamU, 0, sizeof(double) * S, st);  // adjoint of B
            cudaMemsetAsync(a->lamB, 0, sizeof(double) * S, st);  // adjoint of U^n
            double* lo = a->lamA;
            double* ly[2] = {a->lamY0, a->lamY1};
            int flip = 0;
            for (int d = dim - 1; d >= 0; --d) {
                const double* Yin = d > 0 ? Yout[1][d - 1] : nullptr;
                double* lyin = ly[flip];
                rev_dir(B, Yin, An, lo, lyin, a->lamU, a->lamB, d, d == 0, d == dim - 1, d == dim - 1 ? 1 : 0);
                lo = lyin;
                flip ^= 1;
            }
            // stage 1 reversed: the adjoint of B drives it; U^n's adjoint collects in lamB
            cudaMemcpyAsync(a->lamA, a->lamU, sizeof(double) * S, cudaMemcpyDeviceToDevice, st);
            lo = a->lamA;
            for (int d = dim - 1; d >= 0; --d) {
                const double* Yin = d > 0 ? Yout[0][d - 1] : nullptr;
                double* lyin = ly[flip];
                rev_dir(An, Yin, nullptr, lo, lyin, a->lamB, nullptr, d, d == 0, d == dim - 1, 0);
                lo = lyin;
                flip ^= 1;
            }
            cudaMemcpyAsync(a->lamA, a->lamB, sizeof(double) * S, cudaMemcpyDeviceToDevice, st);
        }
    }
    // the initial primitiveToConservative
    k_gen_p2c_rev<<<gblocks(N), kGT, 0, st>>>(PT, fb, a->prim0, a->lamA, grad_prim, mp > 0 ? a->geos : nullptr, npar,
                                              a->nprim);
    ++launches;
    if (mp > 0) {
        k_gen_sum<<<mp, 256, 0, st>>>(a->geos, N, a->gsum);
        ++launches;
        std::vector<double> gs(mp);
        cudaMemcpyAsync(gs.data(), a->gsum, sizeof(double) * mp, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        for (int m = 0; m < P.M; ++m)
            for (int k = 0; k < TJ_MAX_EOS_PARAMS; ++k)
                grad_eos[m * TJ_MAX_EOS_PARAMS + k] = k < npar ? gs[m * npar + k] : 0.0;
    } else {
        for (int k = 0; k < P.M * TJ_MAX_EOS_PARAMS; ++k) grad_eos[k] = 0.0;
    }
    return launches;
}

}  // namespace tj
