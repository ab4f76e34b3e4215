// Adjoint of the FP64 per-timestep update (2-D fluids, stiffened-gas EOS, one
// domain) with a given dt schedule: checkpoint-and-recompute over intervals
// of `stride` steps, then a hand-written reverse of each RK stage.
//
// Forward step n (the reference's main.cpp:145-170 for fluids; dt frozen):
//   S1 = stage(S0), S2 = stage(S1)                     (HLLCadvance, hllc.cpp:579-695)
//   S0' = cleanUpAlpha(S0 / 2 + S2 / 2)                (hllc.cpp:705, main.cpp:170)
// where stage(X) = c2p(C(X) + sum_d dt/dx_d (F_{i-1/2} - F_{i+1/2}) [- alpha S*])
// and the face fluxes F come from the reconstructed states of the stage
// input's primitives. The recompute runs the FP64 kernels themselves
// (fp64_stage), recording the alpha of each reconstructed state after the
// BVD-THINC choice; the reverse of a stage is
//   k_adj_c2p    mu = adjoint of the conserved stage output (c2p reversed)
//   k_adj_face   per face: the flux adjoint dt/dx (mu_right - mu_left) through
//                HLLC, the face-state closures and cleanUpAlpha to the
//                adjoint of the two reconstructed states
//   k_adj_thinc  per cell whose alpha came from its own THINC candidate: the
//                candidate's 3x3-stencil gradient
//   k_adj_gather per cell: adjoint of the stage input (identity, the
//                non-conservative alpha term, the MUSCL and THINC stencils,
//                ghost images folded back onto their source cells)
// Discrete choices are held at their forward values. Alpha values that the
// BVD step takes from the THINC scratch (the reference's stale ULStar/URStar,
// thinc.cpp:138-147,164-165, hllc.cpp:622-623) carry their adjoint back to
// the pass that wrote them, through two adjoint slots per material and cell
// that persist across stages, steps and checkpoint intervals:
//   ULStar is rewritten by every flux pass with the star alpha of the upwind
//   face state (hllc.cpp:406,419-468), so a value read in pass P was written
//   by pass P - 1: k_adj_face adds the slot to that face state's alpha
//   adjoint and clears it;
//   URStar is written only by the THINC right candidate of a mixed cell, so a
//   value read in pass P was written by the last earlier pass in which the
//   cell was mixed: k_adj_thinc adds the slot to the candidate's adjoint there
//   and clears it.
// The reads of a pass are added to the slots (k_adj_scratch) after its
// writes were reversed, and the two directions of a stage are reversed in the
// order d = 1, then d = 0.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "tj_adjoint.cuh"
#include "tj_adjoint_local.h"
#include "tj_device.cuh"

namespace tj {

namespace {

constexpr int NT = 256;
constexpr int NBLK = 152 * 4;  // grid of the kernels that accumulate EOS-parameter adjoints
constexpr int NG = 3 * tja::MM;

struct AG {
    int nx, ny, M, thinc, muscl;
    int lo_bc[2], hi_bc[2];
    double dx[2], beta;
    long long N;
    tja::Eos E;
    int sa, sar, srk, srho, sru, su, sE, sp, ns;
    int NW;  // words of a reconstructed state: alpha[M], rho_k[M], u0, u1, p
    int nl;  // lines of the image arrays: max(nx, ny)
};

__device__ __forceinline__ int mapi(int i, int n, int lo, int hi, bool& refl)
{
    refl = false;
    if (i < 0) {
        if (lo == TJ_BC_REFLECTIVE) { refl = true; return -1 - i; }
        return 0;
    }
    if (i > n - 1) {
        if (hi == TJ_BC_REFLECTIVE) { refl = true; return 2 * n - 1 - i; }
        return n - 1;
    }
    return i;
}

// carried-state word of reconstructed variable q
__device__ __forceinline__ int qword(const AG& G, int q)
{
    if (q < G.M) return G.sa + q;
    if (q < 2 * G.M) return G.srk + q - G.M;
    if (q < 2 * G.M + 2) return G.su + q - 2 * G.M;
    return G.sp;
}

// reconstructed variable q at cell (i, j) + s * o_d (s in -1, 0, 1), ghosts
// mapped, the normal velocity negated in a reflected ghost
__device__ __forceinline__ double qat(const AG& G, const double* X, int i, int j, int d, int s, int q)
{
    bool refl;
    if (d == 0) i = mapi(i + s, G.nx, G.lo_bc[0], G.hi_bc[0], refl);
    else j = mapi(j + s, G.ny, G.lo_bc[1], G.hi_bc[1], refl);
    const double v = X[(long long)qword(G, q) * G.N + i + (long long)G.nx * j];
    return (refl && q == 2 * G.M + d) ? -v : v;
}

__device__ __forceinline__ double& pw(tja::Prim& x, int M, int q)
{
    if (q < M) return x.a[q];
    if (q < 2 * M) return x.rk[q - M];
    if (q < 2 * M + 2) return x.u[q - 2 * M];
    return x.p;
}

// reconstructed state of valid cell (i, j) on side (0 UL, 1 UR) along d
__device__ void face_prim(const AG& G, const double* X, const double* rec, int i, int j, int d, int side, tja::Prim& x)
{
    const long long g = i + (long long)G.nx * j;
    for (int q = 0; q < G.NW; ++q) {
        const double u0 = qat(G, X, i, j, d, 0, q);
        double v = u0;
        if (G.muscl) {
            double l, r;
            tja::muscl_fwd(qat(G, X, i, j, d, -1, q), u0, qat(G, X, i, j, d, 1, q), l, r);
            v = side ? r : l;
        }
        pw(x, G.M, q) = v;
    }
    if (G.thinc)
        for (int m = 0; m < G.M; ++m) x.a[m] = rec[((long long)(d * 2 + side) * G.M + m) * G.N + g];
}

// Adds the block's sum of g to its slot gpart[blockIdx.x][k], k = m (G),
// MM + m (p_ref), 2 MM + m (e_ref).
__device__ void block_add_grad(const tja::GradEos& g, int M, double* gpart)
{
    __shared__ double red[NT / 32][NG];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < NG; ++k) {
        const int m = k % tja::MM, kind = k / tja::MM;
        double v = m >= M ? 0.0 : (kind == 0 ? g.G[m] : (kind == 1 ? g.pr[m] : g.er[m]));
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < NG; ++k) {
            double s = 0.0;
            for (int w = 0; w < NT / 32; ++w) s += red[w][k];
            gpart[(long long)blockIdx.x * NG + k] += s;
        }
}

// ---------------------------------------------------------------------------
// Forward: S0' = cleanUpAlpha(S0 / 2 + S2 / 2), the expression of the FP64
// stage-2 finish (bit for bit).
// ---------------------------------------------------------------------------
__global__ void k_adj_avg(DevParams P, AG G, const double* S0, const double* S2, double* out, DevScalars* scal)
{
    const long long N = G.N;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        for (int w = 0; w < G.ns; ++w) out[w * N + g] = (S0[w * N + g] * (1.0 / 2.0)) + (S2[w * N + g] * (1.0 / 2.0));
        double a[TJ_MAX_MAT];
        for (int m = 0; m < G.M; ++m) a[m] = out[(G.sa + m) * N + g];
        const int e = cleanup_alpha(P, a);
        if (e) atomicCAS(&scal->status, 0, e);
        for (int m = 0; m < G.M; ++m) out[(G.sa + m) * N + g] = a[m];
    }
}

// ---------------------------------------------------------------------------
// Reverse of the average and cleanUpAlpha: lam <- lam_avg / 2 (the S0 part),
// lamA <- lam_avg / 2 (the S2 part).
// ---------------------------------------------------------------------------
__global__ void k_adj_finish(AG G, double* lam, double* lamA, const double* S0, const double* S2)
{
    const long long N = G.N;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        double aavg[tja::MM], la[tja::MM], li[tja::MM];
        for (int m = 0; m < G.M; ++m) {
            aavg[m] = (S0[(G.sa + m) * N + g] * (1.0 / 2.0)) + (S2[(G.sa + m) * N + g] * (1.0 / 2.0));
            la[m] = lam[(G.sa + m) * N + g];
        }
        tja::cleanup_rev(G.M, aavg, la, li);
        for (int w = 0; w < G.ns; ++w) {
            double v = lam[w * N + g];
            if (w >= G.sa && w < G.sa + G.M) v = li[w - G.sa];
            if (w == G.sru + 2 || w == G.su + 2) v = 0.0;
            lam[w * N + g] = 0.5 * v;
            lamA[w * N + g] = 0.5 * v;
        }
    }
}

// ---------------------------------------------------------------------------
// mu = adjoint of the conserved words of a stage output Y, from the adjoint of
// all its carried words (conservativeToPrimitive reversed).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_adj_c2p(AG G, const double* lamY, const double* Y, double* mu, double* gpart)
{
    const long long N = G.N;
    const int M = G.M;
    tja::GradEos gr;
    tja::zero(gr);
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        tja::Cons c;
        tja::Carried l;
        tja::zero(c);
        tja::zero(l);
        for (int m = 0; m < M; ++m) {
            c.a[m] = Y[(G.sa + m) * N + g];
            c.ar[m] = Y[(G.sar + m) * N + g];
            l.a[m] = lamY[(G.sa + m) * N + g];
            l.ar[m] = lamY[(G.sar + m) * N + g];
            l.rk[m] = lamY[(G.srk + m) * N + g];
        }
        for (int r = 0; r < 2; ++r) {
            c.ru[r] = Y[(G.sru + r) * N + g];
            l.ru[r] = lamY[(G.sru + r) * N + g];
            l.u[r] = lamY[(G.su + r) * N + g];
        }
        c.E = Y[G.sE * N + g];
        l.E = lamY[G.sE * N + g];
        l.p = lamY[G.sp * N + g];
        l.rho = lamY[G.srho * N + g];
        tja::Cons o;
        tja::c2p_rev(G.E, c, l, o, gr);
        for (int m = 0; m < M; ++m) {
            mu[(long long)m * N + g] = o.a[m];
            mu[(long long)(M + m) * N + g] = o.ar[m];
        }
        mu[(long long)(2 * M) * N + g] = o.ru[0];
        mu[(long long)(2 * M + 1) * N + g] = o.ru[1];
        mu[(long long)(2 * M + 2) * N + g] = o.E;
    }
    block_add_grad(gr, M, gpart);
}

// ---------------------------------------------------------------------------
// Per face along d: adjoint of the two reconstructed states that meet there.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_adj_face(AG G, int d, const double* X, const double* rec, const double* mu,
                                                 double* lface, double* limg, double* sstar, double dt, double* gpart,
                                                 double* sul)
{
    const int M = G.M, NW = G.NW;
    const long long N = G.N;
    const int nfx = G.nx + (d == 0);
    const long long nf = (long long)nfx * (G.ny + (d == 1));
    const int n = d == 0 ? G.nx : G.ny;
    const double dtdx = dt / G.dx[d];
    tja::GradEos gr;
    tja::zero(gr);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x) {
        const int fi = (int)(f % nfx), fj = (int)(f / nfx);
        const int pos = d == 0 ? fi : fj, line = d == 0 ? fj : fi;
        const bool imgL = pos == 0, imgR = pos == n;
        const bool reflL = imgL && G.lo_bc[d] == TJ_BC_REFLECTIVE, reflR = imgR && G.hi_bc[d] == TJ_BC_REFLECTIVE;
        const int pl = imgL ? 0 : pos - 1, pr = imgR ? n - 1 : pos;
        const int li = d == 0 ? pl : line, lj = d == 0 ? line : pl;
        const int ri = d == 0 ? pr : line, rj = d == 0 ? line : pr;
        const long long gL = li + (long long)G.nx * lj, gR = ri + (long long)G.nx * rj;
        tja::Prim xl, xr;
        face_prim(G, X, rec, li, lj, d, 1, xl);
        face_prim(G, X, rec, ri, rj, d, 0, xr);
        if (reflL) xl.u[d] = -xl.u[d];
        if (reflR) xr.u[d] = -xr.u[d];
        tja::FS L, R;
        tja::face_state_fwd(G.E, xl, G.thinc != 0, L);
        tja::face_state_fwd(G.E, xr, G.thinc != 0, R);
        // flux adjoint: the face adds F to its right cell and subtracts it
        // from its left cell; S* enters as -alpha_right S* + alpha_left S*
        tja::HllcOut lF;
        const bool hasR = pos < n, hasL = pos >= 1;
        const long long cR = hasR ? gR : 0, cL = hasL ? (d == 0 ? (pos - 1) + (long long)G.nx * line
                                                                : line + (long long)G.nx * (pos - 1))
                                                      : 0;
        double lS = 0.0;
        for (int m = 0; m < M; ++m) {
            const double muRa = hasR ? mu[(long long)m * N + cR] : 0.0, muLa = hasL ? mu[(long long)m * N + cL] : 0.0;
            const double muRr = hasR ? mu[(long long)(M + m) * N + cR] : 0.0,
                         muLr = hasL ? mu[(long long)(M + m) * N + cL] : 0.0;
            lF.Fa[m] = dtdx * (muRa - muLa);
            lF.Far[m] = dtdx * (muRr - muLr);
            if (hasR) lS -= X[(G.sa + m) * N + cR] * muRa;
            if (hasL) lS += X[(G.sa + m) * N + cL] * muLa;
        }
        for (int m = M; m < tja::MM; ++m) lF.Fa[m] = lF.Far[m] = 0.0;
        for (int r = 0; r < 2; ++r)
            lF.Fru[r] = dtdx * ((hasR ? mu[(long long)(2 * M + r) * N + cR] : 0.0) -
                                (hasL ? mu[(long long)(2 * M + r) * N + cL] : 0.0));
        lF.FE = dtdx * ((hasR ? mu[(long long)(2 * M + 2) * N + cR] : 0.0) -
                        (hasL ? mu[(long long)(2 * M + 2) * N + cL] : 0.0));
        lF.Ss = dtdx * lS;
        tja::FS lL, lR;
        tja::zero(lL);
        tja::zero(lR);
        const double Ss = tja::hllc_rev(M, L, R, d, lF, lL, lR);
        if (sul && hasR) {
            // this pass wrote the star alpha of the face's upwind state into
            // ULStar at its valid right cell (hllc.cpp:406,419-468): the
            // adjoint that later reads of that slot gathered goes to it
            const double x1 = fabs(L.u[d]) + L.c, x2 = fabs(R.u[d]) + R.c;
            const double SL = -((x1 < x2) ? x2 : x1);
            const bool left = (SL >= 0.0) || (Ss >= 0.0);
            for (int m = 0; m < M; ++m) {
                const double v = sul[(long long)m * N + gR];
                if (left) lL.a[m] += v;
                else lR.a[m] += v;
                sul[(long long)m * N + gR] = 0.0;
            }
        }
        tja::Prim pL, pR;
        tja::zero(pL);
        tja::zero(pR);
        tja::face_state_rev(G.E, xl, G.thinc != 0, lL, pL, gr);
        tja::face_state_rev(G.E, xr, G.thinc != 0, lR, pR, gr);
        if (reflL) pL.u[d] = -pL.u[d];
        if (reflR) pR.u[d] = -pR.u[d];
        for (int q = 0; q < NW; ++q) {
            if (!imgL) lface[((long long)(d * 2 + 1) * NW + q) * N + gL] = pw(pL, M, q);
            else limg[((long long)(d * 2) * NW + q) * G.nl + line] = pw(pL, M, q);
            if (!imgR) lface[((long long)(d * 2) * NW + q) * N + gR] = pw(pR, M, q);
            else limg[((long long)(d * 2 + 1) * NW + q) * G.nl + line] = pw(pR, M, q);
        }
        sstar[f] = Ss;
    }
    block_add_grad(gr, M, gpart);
}

__device__ double thinc_cosh(double x) { return tjm_cosh(x); }
__device__ double thinc_tanh(double x) { return tjm_tanh(x); }
__device__ double thinc_exp(double x) { return tjm_exp(x); }

// ---------------------------------------------------------------------------
// Per cell along d: stencil gradient of each THINC candidate the forward used.
// ---------------------------------------------------------------------------
__global__ void k_adj_thinc(AG G, int d, const double* X, const int* code, const double* lface, const double* limg,
                            double* tcon, double* sur)
{
    const int M = G.M, NW = G.NW;
    const long long N = G.N;
    const int n = d == 0 ? G.nx : G.ny;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        const int cd = code[(long long)d * N + g];
        const int i = (int)(g % G.nx), j = (int)(g / G.nx);
        const int pos = d == 0 ? i : j, line = d == 0 ? j : i;
        for (int m = 0; m < M; ++m) {
            double* tc = tcon + (long long)((d * M + m) * 9) * N + g;
            double s[3][3], ls[3][3];
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c) {
                    bool r0, r1;
                    const int ii = mapi(i + a - 1, G.nx, G.lo_bc[0], G.hi_bc[0], r0);
                    const int jj = mapi(j + c - 1, G.ny, G.lo_bc[1], G.hi_bc[1], r1);
                    s[a][c] = X[(G.sa + m) * N + ii + (long long)G.nx * jj];
                    ls[a][c] = 0.0;
                }
            double cL = 0.0, cR = 0.0;
            const bool mixed = tja::thinc_cand_fwd(s, d, G.beta, G.dx[0], G.dx[1], thinc_cosh, thinc_tanh, thinc_exp,
                                                   cL, cR);
            double lL = 0.0, lR = 0.0;
            if (((cd >> (2 * m)) & 3) == 1) {  // the cell's own candidate, used in this pass
                lL = lface[((long long)(d * 2) * NW + m) * N + g];
                lR = lface[((long long)(d * 2 + 1) * NW + m) * N + g];
                if (pos == n - 1) lL += limg[((long long)(d * 2 + 1) * NW + m) * G.nl + line];
                if (pos == 0) lR += limg[((long long)(d * 2) * NW + m) * G.nl + line];
            }
            if (mixed && sur) {
                // this pass wrote the right candidate into URStar
                // (thinc.cpp:138-147): the adjoint of its later reads
                lR += sur[(long long)m * N + g];
                sur[(long long)m * N + g] = 0.0;
            }
            if (mixed && (lL != 0.0 || lR != 0.0))
                tja::thinc_cand_rev(s, d, G.beta, G.dx[0], G.dx[1], thinc_cosh, thinc_tanh, thinc_exp, lL, lR, ls);
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c) tc[(long long)(a * 3 + c) * N] = ls[a][c];
        }
    }
}

// ---------------------------------------------------------------------------
// Per cell along d: the reconstructed alpha values this pass took from the
// THINC scratch (code 2: UL alpha = ULStar, UR alpha = URStar of the cell)
// add their adjoint to the scratch slots, for the earlier passes that wrote
// those values.
// ---------------------------------------------------------------------------
__global__ void k_adj_scratch(AG G, int d, const int* code, const double* lface, const double* limg, double* sul,
                              double* sur)
{
    const int M = G.M, NW = G.NW;
    const long long N = G.N;
    const int n = d == 0 ? G.nx : G.ny;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        const int cd = code[(long long)d * N + g];
        if (!cd) continue;
        const int i = (int)(g % G.nx), j = (int)(g / G.nx);
        const int pos = d == 0 ? i : j, line = d == 0 ? j : i;
        for (int m = 0; m < M; ++m) {
            if (((cd >> (2 * m)) & 3) != 2) continue;
            double lL = lface[((long long)(d * 2) * NW + m) * N + g];
            double lR = lface[((long long)(d * 2 + 1) * NW + m) * N + g];
            if (pos == n - 1) lL += limg[((long long)(d * 2 + 1) * NW + m) * G.nl + line];
            if (pos == 0) lR += limg[((long long)(d * 2) * NW + m) * G.nl + line];
            sul[(long long)m * N + g] += lL;
            sur[(long long)m * N + g] += lR;
        }
    }
}

// ---------------------------------------------------------------------------
// Per cell: adjoint of the stage input (written, or added to lamX).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_adj_gather(AG G, const double* X, const int* code, const double* lface,
                                                   const double* limg, const double* mu, const double* sstar0,
                                                   const double* sstar1, const double* tcon, double* lamX, double dt,
                                                   int accumulate)
{
    const int M = G.M, NW = G.NW;
    const long long N = G.N;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(g % G.nx), j = (int)(g / G.nx);
        double acc[2 * tja::MM + 3];  // reconstructed variables: alpha, rho_k, u0, u1, p
        for (int q = 0; q < NW; ++q) acc[q] = 0.0;
        // non-conservative alpha term: -dt/dx alpha (S*_{i-1/2} - S*_{i+1/2})
        double dS = 0.0;
        {
            const long long f0 = i + (long long)(G.nx + 1) * j;
            dS += dt / G.dx[0] * (sstar0[f0] - sstar0[f0 + 1]);
            const long long h0 = i + (long long)G.nx * j;
            dS += dt / G.dx[1] * (sstar1[h0] - sstar1[h0 + G.nx]);
        }
        for (int m = 0; m < M; ++m) acc[m] -= dS * mu[(long long)m * N + g];
        // MUSCL: cells ip = pos-1..pos+1 along d read this cell
        for (int d = 0; d < 2; ++d) {
            const int n = d == 0 ? G.nx : G.ny;
            const int pos = d == 0 ? i : j, line = d == 0 ? j : i;
            const int lo = d == 0 ? G.lo_bc[0] : G.lo_bc[1], hi = d == 0 ? G.hi_bc[0] : G.hi_bc[1];
            for (int ip = pos - 1; ip <= pos + 1; ++ip) {
                if (ip < 0 || ip >= n) continue;
                const int ci = d == 0 ? ip : line, cj = d == 0 ? line : ip;
                const long long gi = ci + (long long)G.nx * cj;
                const int cd = G.thinc ? code[(long long)d * N + gi] : 0;
                bool rm, rp;
                const int mm = mapi(ip - 1, n, lo, hi, rm), mp = mapi(ip + 1, n, lo, hi, rp);
                for (int q = 0; q < NW; ++q) {
                    if (q < M && ((cd >> (2 * q)) & 3)) continue;  // alpha from THINC
                    double lul = lface[((long long)(d * 2) * NW + q) * N + gi];
                    double lur = lface[((long long)(d * 2 + 1) * NW + q) * N + gi];
                    if (ip == n - 1) lul += limg[((long long)(d * 2 + 1) * NW + q) * G.nl + line];
                    if (ip == 0) lur += limg[((long long)(d * 2) * NW + q) * G.nl + line];
                    double lum = 0.0, lu0 = lul + lur, lup = 0.0;
                    if (G.muscl) {
                        const double um = qat(G, X, ci, cj, d, -1, q), u0 = qat(G, X, ci, cj, d, 0, q),
                                     up = qat(G, X, ci, cj, d, 1, q);
                        tja::muscl_rev(tja::muscl_branch(um, u0, up), lul, lur, lum, lu0, lup);
                    }
                    const bool nrm = q == 2 * M + d;
                    if (ip == pos) acc[q] += lu0;
                    if (mm == pos) acc[q] += (rm && nrm) ? -lum : lum;
                    if (mp == pos) acc[q] += (rp && nrm) ? -lup : lup;
                }
            }
        }
        // THINC candidates of the 3x3 neighbours that read this cell
        if (G.thinc) {
            for (int d = 0; d < 2; ++d)
                for (int a = -1; a <= 1; ++a)
                    for (int c = -1; c <= 1; ++c) {
                        const int ci = i + a, cj = j + c;
                        if (ci < 0 || ci >= G.nx || cj < 0 || cj >= G.ny) continue;
                        const long long gi = ci + (long long)G.nx * cj;
                        for (int m = 0; m < M; ++m) {
                            // k_adj_thinc wrote every cell's slots (zero where
                            // no candidate of this pass carries an adjoint)
                            for (int oa = 0; oa < 3; ++oa)
                                for (int oc = 0; oc < 3; ++oc) {
                                    bool r0, r1;
                                    if (mapi(ci + oa - 1, G.nx, G.lo_bc[0], G.hi_bc[0], r0) != i) continue;
                                    if (mapi(cj + oc - 1, G.ny, G.lo_bc[1], G.hi_bc[1], r1) != j) continue;
                                    acc[m] += tcon[((long long)((d * M + m) * 9) + oa * 3 + oc) * N + gi];
                                }
                        }
                    }
        }
        // write: identity on the conserved words, acc on the reconstructed ones
        double out[64];
        for (int w = 0; w < G.ns; ++w) out[w] = 0.0;
        for (int m = 0; m < M; ++m) {
            out[G.sa + m] = mu[(long long)m * N + g] + acc[m];
            out[G.sar + m] = mu[(long long)(M + m) * N + g];
            out[G.srk + m] = acc[M + m];
        }
        for (int r = 0; r < 2; ++r) {
            out[G.sru + r] = mu[(long long)(2 * M + r) * N + g];
            out[G.su + r] = acc[2 * M + r];
        }
        out[G.sE] = mu[(long long)(2 * M + 2) * N + g];
        out[G.sp] = acc[2 * M + 2];
        for (int w = 0; w < G.ns; ++w) {
            if (accumulate) lamX[w * N + g] += out[w];
            else lamX[w * N + g] = out[w];
        }
    }
}

// ---------------------------------------------------------------------------
// Reverse of the initial primitiveToConservative: the adjoint of the
// primitives in the layout of tj_set_primitive (alpha[M], rho_k[M], u[3], p).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) k_adj_p2c0(AG G, const double* lam, const double* S0, double* gprim, double* gpart)
{
    const long long N = G.N;
    const int M = G.M;
    tja::GradEos gr;
    tja::zero(gr);
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        tja::Prim x;
        tja::Carried l;
        tja::zero(x);
        tja::zero(l);
        for (int m = 0; m < M; ++m) {
            x.a[m] = S0[(G.sa + m) * N + g];
            x.rk[m] = S0[(G.srk + m) * N + g];
            l.a[m] = lam[(G.sa + m) * N + g];
            l.ar[m] = lam[(G.sar + m) * N + g];
            l.rk[m] = lam[(G.srk + m) * N + g];
        }
        for (int r = 0; r < 2; ++r) {
            x.u[r] = S0[(G.su + r) * N + g];
            l.u[r] = lam[(G.su + r) * N + g];
            l.ru[r] = lam[(G.sru + r) * N + g];
        }
        x.p = S0[G.sp * N + g];
        l.E = lam[G.sE * N + g];
        l.p = lam[G.sp * N + g];
        l.rho = lam[G.srho * N + g];
        tja::Prim lx;
        tja::p2c_state_rev(G.E, x, l, lx, gr);
        int w = 0;
        for (int m = 0; m < M; ++m) gprim[(long long)(w++) * N + g] = lx.a[m];
        for (int m = 0; m < M; ++m) gprim[(long long)(w++) * N + g] = lx.rk[m];
        gprim[(long long)(w++) * N + g] = lx.u[0];
        gprim[(long long)(w++) * N + g] = lx.u[1];
        gprim[(long long)(w++) * N + g] = 0.0;  // w stays zero in 2-D
        gprim[(long long)(w++) * N + g] = lx.p;
    }
    block_add_grad(gr, M, gpart);
}

__global__ void k_adj_gsum(const double* gpart, int nblk, double* out)
{
    const int k = threadIdx.x;
    if (k >= NG) return;
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += gpart[(long long)b * NG + k];
    out[k] = s;
}

inline int nb(long long n) { return (int)std::min<long long>((n + NT - 1) / NT, 152 * 16); }

AG make_ag(const DevParams& P, const DevDomain& D)
{
    AG G;
    std::memset(&G, 0, sizeof G);
    G.nx = D.n[0];
    G.ny = D.n[1];
    G.M = P.M;
    G.thinc = P.thinc;
    G.muscl = P.muscl;
    for (int d = 0; d < 2; ++d) {
        G.lo_bc[d] = P.lo_bc[d];
        G.hi_bc[d] = P.hi_bc[d];
        G.dx[d] = D.dx[d];
    }
    G.beta = P.beta;
    G.N = (long long)D.n[0] * D.n[1];
    G.E.M = P.M;
    for (int m = 0; m < tja::MM; ++m) {
        const bool on = m < P.M;
        G.E.G[m] = on ? P.prm[m][0] - 1.0 : 1.0;
        G.E.pr[m] = on ? P.prm[m][1] : 0.0;
        G.E.er[m] = on ? P.prm[m][2] : 0.0;
    }
    G.sa = P.S_ALPHA;
    G.sar = P.S_ARHO;
    G.srk = P.S_RHOK;
    G.srho = P.S_RHO;
    G.sru = P.S_RHOU;
    G.su = P.S_VEL;
    G.sE = P.S_E;
    G.sp = P.S_P;
    G.ns = P.NS;
    G.NW = 2 * P.M + 3;
    G.nl = std::max(D.n[0], D.n[1]);
    return G;
}

}  // namespace

struct AdjState {
    int nsteps = 0, stride = 0, nck = 0;
    long long N = 0;
    int M = 0, ns = 0;
    std::vector<double> dt;
    size_t ck_words = 0;
    double* ck = nullptr;   // checkpoints: state, ulstar, urstar, gstar x, gstar y
    double* seg = nullptr;  // 3 stride + 1 states of the interval being reversed
    double* rec = nullptr;  // reconstruction records, 2 stride stages
    int* code = nullptr;
    double *lam = nullptr, *lamA = nullptr, *lamB = nullptr, *mu = nullptr, *lface = nullptr, *limg = nullptr;
    double *sstar = nullptr, *tcon = nullptr, *gpart = nullptr, *gsum = nullptr;
    double *sul = nullptr, *sur = nullptr;  // adjoint of the ULStar / URStar alpha slots
    size_t bytes = 0;
    size_t cap_ck = 0, cap_seg = 0;  // allocated checkpoint / interval capacity (in checkpoints, in steps)
    long long capN = -1;
    int capM = -1;
};

const char* adj_unsupported(const DevParams& P, int ndom)
{
    if (P.dim != 2) return "the adjoint covers 2-D domains";
    if (P.solid || P.plastic) return "the adjoint covers fluids";
    if (P.radial) return "the adjoint covers planar geometry (RADIAL = 0)";
    if (P.M > tja::MM) return "the adjoint covers up to 4 materials";
    for (int m = 0; m < P.M; ++m)
        if (P.eos[m] != TJ_EOS_MIEGRUNEISEN) return "the adjoint covers the stiffened-gas Mie-Gruneisen EOS";
    if (ndom != 1) return "the adjoint covers one domain";
    return nullptr;
}

AdjState* adj_create() { return new AdjState(); }

static void free_all(AdjState* a)
{
    double* ds[] = {a->ck, a->seg, a->rec, a->lam, a->lamA, a->lamB, a->mu, a->lface, a->limg, a->sstar, a->tcon,
                    a->gpart, a->gsum, a->sul, a->sur};
    for (double* p : ds)
        if (p) cudaFree(p);
    if (a->code) cudaFree(a->code);
    a->ck = a->seg = a->rec = a->lam = a->lamA = a->lamB = a->mu = a->lface = a->limg = a->sstar = a->tcon = nullptr;
    a->gpart = a->gsum = nullptr;
    a->sul = a->sur = nullptr;
    a->code = nullptr;
    a->bytes = 0;
    a->cap_ck = a->cap_seg = 0;
    a->capN = -1;
}

void adj_destroy(AdjState* a)
{
    if (!a) return;
    free_all(a);
    delete a;
}

size_t adj_bytes(const AdjState* a) { return a ? a->bytes : 0; }

template <typename T>
static bool dalloc(AdjState* a, T** p, size_t n)
{
    if (cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) return false;
    a->bytes += sizeof(T) * n;
    return true;
}

// (Re)allocates what a run of nsteps with this stride needs.
static int ensure(AdjState* a, const DevParams& P, const Fp64Bufs& b, const DevDomain& D, int nsteps, int stride)
{
    const long long N = (long long)D.n[0] * D.n[1];
    const int M = P.M, ns = P.NS;
    const size_t nf0 = (size_t)(D.n[0] + 1) * D.n[1], nf1 = (size_t)D.n[0] * (D.n[1] + 1);
    const size_t ck_words = (size_t)ns * N + 2 * (size_t)M * N + (size_t)M * (nf0 + nf1);
    const size_t nck = (size_t)((nsteps + stride - 1) / stride);
    if (a->capN == N && a->capM == M && a->cap_ck >= nck && a->cap_seg >= (size_t)stride) {
        a->ck_words = ck_words;
        return TJ_OK;
    }
    free_all(a);
    const size_t NW = 2 * M + 3, nl = std::max(D.n[0], D.n[1]);
    bool ok = dalloc(a, &a->ck, nck * ck_words) && dalloc(a, &a->seg, (size_t)(3 * stride + 1) * ns * N) &&
              dalloc(a, &a->rec, (size_t)2 * stride * 4 * M * N) && dalloc(a, &a->code, (size_t)2 * stride * 2 * N) &&
              dalloc(a, &a->lam, (size_t)ns * N) && dalloc(a, &a->lamA, (size_t)ns * N) &&
              dalloc(a, &a->lamB, (size_t)ns * N) && dalloc(a, &a->mu, NW * N) && dalloc(a, &a->lface, 4 * NW * N) &&
              dalloc(a, &a->limg, 4 * NW * nl) && dalloc(a, &a->sstar, nf0 + nf1) &&
              dalloc(a, &a->tcon, (size_t)2 * M * 9 * N) && dalloc(a, &a->gpart, (size_t)NBLK * NG) &&
              dalloc(a, &a->gsum, NG) && dalloc(a, &a->sul, (size_t)M * N) && dalloc(a, &a->sur, (size_t)M * N);
    if (!ok) {
        free_all(a);
        return TJ_ERR_CUDA;
    }
    a->ck_words = ck_words;
    a->cap_ck = nck;
    a->cap_seg = stride;
    a->capN = N;
    a->capM = M;
    (void)b;
    return TJ_OK;
}

static void copy_scratch(const DevParams& P, const Fp64Bufs& b, const DevDomain& D, double* ck, bool save,
                         cudaStream_t st)
{
    const long long N = (long long)D.n[0] * D.n[1];
    const size_t nf0 = (size_t)(D.n[0] + 1) * D.n[1], nf1 = (size_t)D.n[0] * (D.n[1] + 1);
    const int M = P.M;
    double* p = ck + (size_t)P.NS * N;
    struct {
        double* dev;
        size_t n;
    } parts[4] = {{b.ulstar, (size_t)M * N}, {b.urstar, (size_t)M * N}, {b.gstar[0], M * nf0}, {b.gstar[1], M * nf1}};
    for (auto& q : parts) {
        if (!q.dev) continue;  // no THINC scratch without THINC
        if (save) cudaMemcpyAsync(p, q.dev, sizeof(double) * q.n, cudaMemcpyDeviceToDevice, st);
        else cudaMemcpyAsync(q.dev, p, sizeof(double) * q.n, cudaMemcpyDeviceToDevice, st);
        p += q.n;
    }
}

long long adj_forward(AdjState* a, const DevParams& P, const Fp64Bufs& b, const DevDomain& D, const double* dt,
                      int nsteps, int stride, cudaStream_t st)
{
    if (nsteps < 1 || stride < 1) return TJ_ERR_ARG;
    stride = std::min(stride, nsteps);
    int e = ensure(a, P, b, D, nsteps, stride);
    if (e) return e;
    a->nsteps = nsteps;
    a->stride = stride;
    a->nck = (nsteps + stride - 1) / stride;
    a->N = (long long)D.n[0] * D.n[1];
    a->M = P.M;
    a->ns = P.NS;
    a->dt.assign(dt, dt + nsteps);
    const AG G = make_ag(P, D);
    Fp64Bufs bb = b;
    bb.rec = nullptr;
    bb.rec_code = nullptr;
    long long launches = 0;
    const size_t sw = (size_t)P.NS * a->N;
    for (int n = 0; n < nsteps; ++n) {
        if (n % stride == 0) {
            double* ck = a->ck + (size_t)(n / stride) * a->ck_words;
            cudaMemcpyAsync(ck, b.A, sizeof(double) * sw, cudaMemcpyDeviceToDevice, st);
            copy_scratch(P, b, D, ck, true, st);
        }
        launches += fp64_set_dt(bb, dt[n], st);
        launches += fp64_stage(P, bb, b.A, b.B, 0, st);
        launches += fp64_stage(P, bb, b.B, b.C, 0, st);
        k_adj_avg<<<nb(a->N), NT, 0, st>>>(P, G, b.A, b.C, b.A, b.scal);
        launches += 1;
    }
    return launches;
}

long long adj_backward(AdjState* a, const DevParams& P, const Fp64Bufs& b, const DevDomain& D, const double* lam_final,
                       double* grad_prim, double* grad_eos, cudaStream_t st)
{
    if (!a || a->nck == 0 || a->N != (long long)D.n[0] * D.n[1]) return TJ_ERR_STATE;
    const AG G = make_ag(P, D);
    const long long N = a->N;
    const int M = P.M, ns = P.NS;
    const size_t sw = (size_t)ns * N;
    const size_t nf0 = (size_t)(D.n[0] + 1) * D.n[1];
    long long launches = 0;
    cudaMemcpyAsync(a->lam, lam_final, sizeof(double) * sw, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(a->gpart, 0, sizeof(double) * NBLK * NG, st);
    cudaMemsetAsync(a->sul, 0, sizeof(double) * M * N, st);
    cudaMemsetAsync(a->sur, 0, sizeof(double) * M * N, st);
    auto S = [&](int k, int which) { return a->seg + (size_t)(3 * k + which) * sw; };
    const size_t recw = (size_t)4 * M * N;
    for (int s = a->nck - 1; s >= 0; --s) {
        const int n0 = s * a->stride, n1 = std::min(n0 + a->stride, a->nsteps), K = n1 - n0;
        const double* ck = a->ck + (size_t)s * a->ck_words;
        cudaMemcpyAsync(S(0, 0), ck, sizeof(double) * sw, cudaMemcpyDeviceToDevice, st);
        copy_scratch(P, b, D, const_cast<double*>(ck), false, st);
        // recompute the interval, recording the reconstructions
        for (int k = 0; k < K; ++k) {
            launches += fp64_set_dt(b, a->dt[n0 + k], st);
            for (int stage = 0; stage < 2; ++stage) {
                Fp64Bufs bb = b;
                bb.rec = a->rec + (size_t)(2 * k + stage) * recw;
                bb.rec_code = a->code + (size_t)(2 * k + stage) * 2 * N;
                launches += fp64_stage(P, bb, S(k, stage), S(k, stage + 1), 0, st);
            }
            k_adj_avg<<<nb(N), NT, 0, st>>>(P, G, S(k, 0), S(k, 2), S(k + 1, 0), b.scal);
            launches += 1;
        }
        // reverse it
        for (int k = K - 1; k >= 0; --k) {
            const double dtn = a->dt[n0 + k];
            k_adj_finish<<<nb(N), NT, 0, st>>>(G, a->lam, a->lamA, S(k, 0), S(k, 2));
            launches += 1;
            for (int stage = 1; stage >= 0; --stage) {
                const double* X = S(k, stage);
                const double* Y = S(k, stage + 1);
                const double* lamY = stage == 1 ? a->lamA : a->lamB;
                double* lamX = stage == 1 ? a->lamB : a->lam;
                const double* rec = a->rec + (size_t)(2 * k + stage) * recw;
                const int* code = a->code + (size_t)(2 * k + stage) * 2 * N;
                k_adj_c2p<<<NBLK, NT, 0, st>>>(G, lamY, Y, a->mu, a->gpart);
                launches += 1;
                // the stage's passes in reverse order (d = 1, then d = 0): each
                // pass's scratch writes are reversed before its reads
                for (int d = 1; d >= 0; --d) {
                    k_adj_face<<<NBLK, NT, 0, st>>>(G, d, X, rec, a->mu, a->lface, a->limg, a->sstar + (d ? nf0 : 0),
                                                    dtn, a->gpart, P.thinc ? a->sul : nullptr);
                    launches += 1;
                    if (P.thinc) {
                        k_adj_thinc<<<nb(N), NT, 0, st>>>(G, d, X, code, a->lface, a->limg, a->tcon, a->sur);
                        k_adj_scratch<<<nb(N), NT, 0, st>>>(G, d, code, a->lface, a->limg, a->sul, a->sur);
                        launches += 2;
                    }
                }
                k_adj_gather<<<nb(N), NT, 0, st>>>(G, X, code, a->lface, a->limg, a->mu, a->sstar, a->sstar + nf0,
                                                   a->tcon, lamX, dtn, stage == 0 ? 1 : 0);
                launches += 1;
            }
        }
    }
    // the first interval's S(0, 0) is the initial state
    k_adj_p2c0<<<NBLK, NT, 0, st>>>(G, a->lam, a->seg, grad_prim, a->gpart);
    k_adj_gsum<<<1, 32, 0, st>>>(a->gpart, NBLK, a->gsum);
    launches += 2;
    double g[NG];
    cudaMemcpyAsync(g, a->gsum, sizeof g, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    for (int m = 0; m < M; ++m) {
        for (int k = 0; k < TJ_MAX_EOS_PARAMS; ++k) grad_eos[m * TJ_MAX_EOS_PARAMS + k] = 0.0;
        grad_eos[m * TJ_MAX_EOS_PARAMS + 0] = g[m];                // params[0]: G = params[0] - 1
        grad_eos[m * TJ_MAX_EOS_PARAMS + 1] = g[tja::MM + m];      // params[1]: p_ref
        grad_eos[m * TJ_MAX_EOS_PARAMS + 2] = g[2 * tja::MM + m];  // params[2]: e_ref
    }
    return launches;
}

}  // namespace tj
