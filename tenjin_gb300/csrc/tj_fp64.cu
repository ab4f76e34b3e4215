// FP64 reference-faithful kernels of Tenjin's per-timestep update.
//
// One RK stage (HLLCadvance, hllc.cpp:579-695) is, per direction d:
//   k_recon   per cell : MUSCL (hllc.cpp:541-575), BVD-THINC (thinc.cpp:67-208),
//                        cleanUpAlpha of the reconstructed states (hllc.cpp:628-629),
//                        primitiveToConservative + getSoundSpeed (634-638)
//   k_flux    per face : HLLC (hllc.cpp:384-487) or 5-wave (133-380)
//   k_update  per cell : update (hllc.cpp:493-523); after the last direction
//                        conservativeToPrimitive (689), and at the end of the
//                        second stage the RK2 average (705), plasticUpdate,
//                        cleanUpV, cleanUpAlpha and the NaN check
//                        (main.cpp:145-187).
// Ghost cells are never stored: a read outside a domain maps the index back
// (foextrap: nearest cell; reflect: mirror, negating the normal velocity and
// momentum), which is what the reference's FillDomainBoundary and
// FillBoundary calls leave in the ghost cells (main.cpp:124-126,
// hllc.cpp:642-646,690-691).
#include <cuda_runtime.h>

#include "tj_device.cuh"
#include "tj_fp64.cuh"

namespace tj {

static constexpr int kThreads = 256;

static inline int nblocks(long long n, int cap = 152 * 16)
{
    long long b = (n + kThreads - 1) / kThreads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

__device__ __forceinline__ int find_dom(const DevDomain* doms, int ndom, long long g)
{
    int lo = 0, hi = ndom - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (doms[mid].off <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int find_dom_face(const DevDomain* doms, int ndom, int d, long long f)
{
    int lo = 0, hi = ndom - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (doms[mid].foff[d] <= f) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void set_status(DevScalars* s, int code)
{
    atomicCAS(&s->status, 0, code);
}

// Map (i,j,k), possibly outside the domain, to a valid cell; refl[d] = 1 when
// direction d reflected.
__device__ __forceinline__ long long map_cell(const DevParams& P, const DevDomain& D, int i, int j, int k, int* refl)
{
    int ijk[3] = {i, j, k};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        refl[d] = 0;
        if (d >= P.dim) continue;
        int n = D.n[d];
        if (ijk[d] < 0) {
            if (P.lo_bc[d] == TJ_BC_REFLECTIVE) { ijk[d] = -1 - ijk[d]; refl[d] = 1; }
            else ijk[d] = 0;
        } else if (ijk[d] > n - 1) {
            if (P.hi_bc[d] == TJ_BC_REFLECTIVE) { ijk[d] = 2 * n - 1 - ijk[d]; refl[d] = 1; }
            else ijk[d] = n - 1;
        }
    }
    return D.off + ijk[0] + (long long)D.n[0] * (ijk[1] + (long long)D.n[1] * ijk[2]);
}

__device__ __forceinline__ long long face_index(const DevDomain& D, int d, int i, int j, int k)
{
    int nf0 = D.n[0] + (d == 0), nf1 = D.n[1] + (d == 1);
    return D.foff[d] + i + (long long)nf0 * (j + (long long)nf1 * k);
}

// Carried-state load with the reflect_odd sign applied.
__device__ inline void load_state(const DevParams& P, const double* X, long long nt, long long g, const int* refl,
                                  CellS& c)
{
    for (int m = 0; m < P.M; ++m) {
        c.alpha[m] = X[(P.S_ALPHA + m) * nt + g];
        c.arho[m] = X[(P.S_ARHO + m) * nt + g];
        c.rhok[m] = X[(P.S_RHOK + m) * nt + g];
    }
    c.rho = X[P.S_RHO * nt + g];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        double u = X[(P.S_VEL + r) * nt + g], ru = X[(P.S_RHOU + r) * nt + g];
        if (refl && refl[r]) { u = -u; ru = -ru; }
        c.vel[r] = u;
        c.rhou[r] = ru;
    }
    c.E = X[P.S_E * nt + g];
    c.p = X[P.S_P * nt + g];
    c.hj2 = 0.0;
    if (P.solid) {
#pragma unroll
        for (int q = 0; q < 9; ++q) c.V[q] = X[(P.S_V + q) * nt + g];
        c.hj2 = X[P.S_HJ2 * nt + g];
    }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) {
            c.eps[m] = X[(P.S_EPS + m) * nt + g];
            c.are[m] = X[(P.S_ARE + m) * nt + g];
        }
}

__device__ inline void store_state(const DevParams& P, double* X, long long nt, long long g, const CellS& c)
{
    for (int m = 0; m < P.M; ++m) {
        X[(P.S_ALPHA + m) * nt + g] = c.alpha[m];
        X[(P.S_ARHO + m) * nt + g] = c.arho[m];
        X[(P.S_RHOK + m) * nt + g] = c.rhok[m];
    }
    X[P.S_RHO * nt + g] = c.rho;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        X[(P.S_VEL + r) * nt + g] = c.vel[r];
        X[(P.S_RHOU + r) * nt + g] = c.rhou[r];
    }
    X[P.S_E * nt + g] = c.E;
    X[P.S_P * nt + g] = c.p;
    if (P.solid) {
#pragma unroll
        for (int q = 0; q < 9; ++q) X[(P.S_V + q) * nt + g] = c.V[q];
        X[P.S_HJ2 * nt + g] = c.hj2;
    }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) {
            X[(P.S_EPS + m) * nt + g] = c.eps[m];
            X[(P.S_ARE + m) * nt + g] = c.are[m];
        }
}

__device__ inline void store_face(const DevParams& P, double* F, long long nt, long long g, const CellS& c)
{
    for (int m = 0; m < P.M; ++m) {
        F[(P.F_ALPHA + m) * nt + g] = c.alpha[m];
        F[(P.F_ARHO + m) * nt + g] = c.arho[m];
    }
    F[P.F_RHO * nt + g] = c.rho;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        F[(P.F_RHOU + r) * nt + g] = c.rhou[r];
        F[(P.F_VEL + r) * nt + g] = c.vel[r];
    }
    F[P.F_E * nt + g] = c.E;
    F[P.F_P * nt + g] = c.p;
    F[P.F_A * nt + g] = c.a;
    if (P.solid) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            F[(P.F_SIGMA + q) * nt + g] = c.sigma[q];
            F[(P.F_V + q) * nt + g] = c.V[q];
        }
    }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) F[(P.F_ARE + m) * nt + g] = c.are[m];
}

__device__ inline void load_face(const DevParams& P, const double* F, long long nt, long long g, int oddir, CellS& c)
{
    for (int m = 0; m < P.M; ++m) {
        c.alpha[m] = F[(P.F_ALPHA + m) * nt + g];
        c.arho[m] = F[(P.F_ARHO + m) * nt + g];
        c.rhok[m] = 0.0;
    }
    c.rho = F[P.F_RHO * nt + g];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        double u = F[(P.F_VEL + r) * nt + g], ru = F[(P.F_RHOU + r) * nt + g];
        if (r == oddir) { u = -u; ru = -ru; }
        c.vel[r] = u;
        c.rhou[r] = ru;
    }
    c.E = F[P.F_E * nt + g];
    c.p = F[P.F_P * nt + g];
    c.a = F[P.F_A * nt + g];
    c.hj2 = 0.0;
    if (P.solid) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            c.sigma[q] = F[(P.F_SIGMA + q) * nt + g];
            c.V[q] = F[(P.F_V + q) * nt + g];
        }
    } else {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int q = 0; q < 3; ++q) c.sigma[3 * r + q] = -c.p * (double)(r == q);  // stressTensor, fluid
    }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) c.are[m] = F[(P.F_ARE + m) * nt + g];
}

__device__ __forceinline__ double vanleer(double r)  // hllc.cpp:527-537
{
    if (r <= 0.0) return 0.0;
    double a = 2.0 / (1.0 + r), b = 2.0 * r / (1.0 + r);
    return (b < a) ? b : a;
}

__device__ __forceinline__ void muscl1(double um, double u0, double up, double& l, double& r)  // hllc.cpp:557-568
{
    double rr = (u0 - um) / (up - u0);
    if (isinf(rr) || isnan(rr)) rr = 0.0;
    double grad = vanleer(rr) * 0.5 * (up - um);
    l = u0 - 0.5 * grad;
    r = u0 + 0.5 * grad;
}

// One carried word at a possibly-ghost cell.
__device__ __forceinline__ double gv(const DevParams& P, const DevDomain& D, const double* X, long long nt, int word,
                                     int i, int j, int k)
{
    int refl[3];
    long long g = map_cell(P, D, i, j, k, refl);
    double v = X[word * nt + g];
    for (int d = 0; d < P.dim; ++d)
        if (refl[d] && (word == P.S_VEL + d || word == P.S_RHOU + d)) v = -v;
    return v;
}

// ---------------------------------------------------------------------------
// BVD-THINC candidate of one cell (thinc.cpp:67-147).
// ---------------------------------------------------------------------------
struct ThincCand {
    int mixed[TJ_MAX_MAT];
    double L[TJ_MAX_MAT], R[TJ_MAX_MAT];
    int flag;
};

__device__ inline double youngs(const DevParams& P, const DevDomain& D, const double* X, long long nt, int m, int i,
                                int j, int k, int d)  // thinc.cpp:28-53
{
    int a = P.S_ALPHA + m;
#define NB(di, dj) gv(P, D, X, nt, a, i + (di), j + (dj), k)
    double nx = -1.0 / (8.0 * D.dx[0]) * (NB(1, 1) + 2.0 * NB(1, 0) + NB(1, -1) - NB(-1, 1) - 2.0 * NB(-1, 0) - NB(-1, -1));
    double ny = -1.0 / (8.0 * D.dx[1]) * (NB(1, 1) + 2.0 * NB(0, 1) + NB(-1, 1) - NB(-1, -1) - 2.0 * NB(0, -1) - NB(1, -1));
#undef NB
    double norm = sqrt(nx * nx + ny * ny);
    if (norm < 1E-20) return 0;
    return d == 0 ? fabs(nx / norm) : fabs(ny / norm);
}

__device__ inline void thinc_cand(const DevParams& P, const DevDomain& D, const double* X, long long nt, int i, int j,
                                  int k, int d, ThincCand& t)
{
    const double eps = 1E-20, beta0 = P.beta;
    int o[3] = {0, 0, 0};
    o[d] = 1;
    t.flag = 0;
    for (int m = 0; m < P.M; ++m) {
        int a = P.S_ALPHA + m;
        double aL = gv(P, D, X, nt, a, i - o[0], j - o[1], k - o[2]);
        double aR = gv(P, D, X, nt, a, i + o[0], j + o[1], k + o[2]);
        double a0 = gv(P, D, X, nt, a, i, j, k);
        double mn = (aR < aL) ? aR : aL;
        double mx = ((aL < aR) ? aR : aL) - mn;
        double theta = (double)((0.0 < aR - aL) - (aR - aL < 0.0));
        double C = (mx < eps) ? 0.0 : (a0 - mn + eps) / (mx + eps);
        double delta = 1E-4;
        int mixed = (C > delta) && (C < (0.999999 - delta)) && ((aR - a0) * (a0 - aL) >= 0.0);
        t.mixed[m] = mixed;
        t.flag = mixed;  // the last material wins (thinc.cpp:110-114)
        t.L[m] = 0.0;
        t.R[m] = 0.0;
        if (mixed) {
            double nvc = (P.dim == 2) ? youngs(P, D, X, nt, m, i, j, k, d) : 1.0;
            double beta = nvc * beta0 + 0.01;
            double coshB = tjm_cosh(beta), tanhB = tjm_tanh(beta);
            double B = tjm_exp(theta * beta * ((2.0 * C) - 1.0));
            double A = ((B / coshB) - 1.0) / tanhB;
            t.R[m] = mn + (mx / 2.0) * (1.0 + theta * ((tanhB + A) / (1.0 + A * tanhB)));
            t.L[m] = mn + (mx / 2.0) * (1.0 + theta * A);
        }
    }
}

// ---------------------------------------------------------------------------
// Reconstruction of one direction.
// ---------------------------------------------------------------------------
__global__ void k_recon(DevParams P, Fp64Bufs b, const double* __restrict__ X, int d)
{
    if (b.scal->done) return;
    const long long nt = b.ntot;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        const int q = find_dom(b.doms, b.ndom, g);
        const DevDomain D = b.doms[q];
        long long l = g - D.off;
        int i = (int)(l % D.n[0]), j = (int)((l / D.n[0]) % D.n[1]), k = (int)(l / ((long long)D.n[0] * D.n[1]));
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int rm[3], rp[3];
        long long gm = map_cell(P, D, i - o[0], j - o[1], k - o[2], rm);
        long long gp = map_cell(P, D, i + o[0], j + o[1], k + o[2], rp);
        CellS um, u0, up, L, R;
        load_state(P, X, nt, gm, rm, um);
        load_state(P, X, nt, g, nullptr, u0);
        load_state(P, X, nt, gp, rp, up);
        L = u0;
        R = u0;
        if (P.muscl) {  // MUSCLextrapolate over the primitive list
            for (int m = 0; m < P.M; ++m) {
                muscl1(um.alpha[m], u0.alpha[m], up.alpha[m], L.alpha[m], R.alpha[m]);
                muscl1(um.rhok[m], u0.rhok[m], up.rhok[m], L.rhok[m], R.rhok[m]);
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) muscl1(um.vel[r], u0.vel[r], up.vel[r], L.vel[r], R.vel[r]);
            muscl1(um.p, u0.p, up.p, L.p, R.p);
            if (P.solid)
#pragma unroll
                for (int qq = 0; qq < 9; ++qq) muscl1(um.V[qq], u0.V[qq], up.V[qq], L.V[qq], R.V[qq]);
            if (P.plastic)
                for (int m = 0; m < P.M; ++m) muscl1(um.eps[m], u0.eps[m], up.eps[m], L.eps[m], R.eps[m]);
        }
        int reps = 0;
        if (P.thinc) {
            const int* bx = b.boxes + 6 * (D.box_off + b.cell_box[g]);
            int idx[3] = {i, j, k};
            const int in_m = idx[d] - 1 >= bx[d], in_p = idx[d] + 1 <= bx[3 + d];
            reps = D.nbox - b.cell_box[g];
            ThincCand tc, tm, tp;
            thinc_cand(P, D, X, nt, i, j, k, d, tc);
            if (in_m) thinc_cand(P, D, X, nt, i - o[0], j - o[1], k - o[2], d, tm);
            if (in_p) thinc_cand(P, D, X, nt, i + o[0], j + o[1], k + o[2], d, tp);
            const long long gmm = D.off + (i - o[0]) + (long long)D.n[0] * ((j - o[1]) + (long long)D.n[1] * (k - o[2]));
            const long long gpp = D.off + (i + o[0]) + (long long)D.n[0] * ((j + o[1]) + (long long)D.n[1] * (k + o[2]));
            int code = 0;
            for (int m = 0; m < P.M; ++m) {
                const int a = P.S_ALPHA + m;
                double urm, ulp, trm, tlp;
                // UR.left / UL.right: MUSCL value inside the box, stage input in a ghost.
                if (in_m) {
                    double l_, r_;
                    muscl1(gv(P, D, X, nt, a, i - 2 * o[0], j - 2 * o[1], k - 2 * o[2]), um.alpha[m], u0.alpha[m], l_, r_);
                    urm = r_;
                    trm = tm.mixed[m] ? tm.R[m] : b.urstar[(long long)m * nt + gmm];
                } else {
                    urm = um.alpha[m];
                    trm = 0.0;  // URStar ghosts are never written
                }
                if (in_p) {
                    double l_, r_;
                    muscl1(u0.alpha[m], up.alpha[m], gv(P, D, X, nt, a, i + 2 * o[0], j + 2 * o[1], k + 2 * o[2]), l_, r_);
                    ulp = l_;
                    tlp = tp.mixed[m] ? tp.L[m] : b.ulstar[(long long)m * nt + gpp];
                } else {
                    ulp = up.alpha[m];
                    // ULStar's ghost at the box's hi+1 face: star alpha of the last flux pass along d
                    tlp = b.gstar[d][(long long)m * b.nftot[d] + face_index(D, d, i + o[0], j + o[1], k + o[2])];
                }
                double tpl = tc.mixed[m] ? tc.L[m] : b.ulstar[(long long)m * nt + g];
                double tpr = tc.mixed[m] ? tc.R[m] : b.urstar[(long long)m * nt + g];
                double upl = L.alpha[m], upr = R.alpha[m];
#define MN(x, y) (((y) < (x)) ? (y) : (x))
#define TBV(PL, PR)                                                                                          \
    MN(MN(fabs(urm - (PL)) + fabs((PR)-ulp), fabs(trm - (PL)) + fabs((PR)-tlp)),                            \
       MN(fabs(urm - (PL)) + fabs((PR)-tlp), fabs(trm - (PL)) + fabs((PR)-ulp)))
                double tbvm = TBV(upl, upr);
                double tbvt = TBV(tpl, tpr);
#undef TBV
#undef MN
                if (tc.flag && tbvt < tbvm) {
                    L.alpha[m] = tpl;
                    R.alpha[m] = tpr;
                    code |= (tc.mixed[m] ? 1 : 2) << (2 * m);
                }
            }
            if (b.rec) {
                for (int m = 0; m < P.M; ++m) {
                    b.rec[((long long)(d * 2) * P.M + m) * nt + g] = L.alpha[m];
                    b.rec[((long long)(d * 2 + 1) * P.M + m) * nt + g] = R.alpha[m];
                }
                b.rec_code[(long long)d * nt + g] = code;
            }
            // THINC pass 1 writes its candidates into the persistent scratch.
            for (int m = 0; m < P.M; ++m)
                if (tc.mixed[m]) {
                    b.ulstar[(long long)m * nt + g] = tc.L[m];
                    b.urstar[(long long)m * nt + g] = tc.R[m];
                }
        }
        // cleanUpAlpha of UL and UR: nbox-b times for box b, the closures see
        // the first (hllc.cpp:628-638).
        for (int side = 0; side < 2; ++side) {
            CellS& S = side ? R : L;
            if (reps > 0) {
                int e = cleanup_alpha(P, S.alpha);
                if (e) set_status(b.scal, e);
            }
            p2c(P, S);
            S.a = sound_speed(P, S);
            for (int r = 1; r < reps; ++r) {
                double before[TJ_MAX_MAT];
                for (int m = 0; m < P.M; ++m) before[m] = S.alpha[m];
                int e = cleanup_alpha(P, S.alpha);
                if (e) set_status(b.scal, e);
                bool same = true;
                for (int m = 0; m < P.M; ++m)
                    same &= (__double_as_longlong(before[m]) == __double_as_longlong(S.alpha[m]));
                if (same) break;
            }
        }
        store_face(P, b.UL, nt, g, L);
        store_face(P, b.UR, nt, g, R);
    }
}

// ---------------------------------------------------------------------------
// Riemann solvers (hllc.cpp:1-487, flux.cpp:5-47).
// ---------------------------------------------------------------------------
__device__ inline void star_state(const DevParams& P, const CellS& U, CellS& Us, double SK, double Ss, int d)  // :12-73
{
    const double tol = 1E-20;
    double ud = U.vel[d];
    double mult = (fabs((Ss - ud) / Ss) < tol ? 1.0 : (SK - ud) / (SK - Ss));
    Us.rho = 0.0;
    for (int m = 0; m < P.M; ++m) {
        Us.alpha[m] = U.alpha[m];
        Us.arho[m] = mult * U.arho[m];
        Us.rhok[m] = Us.arho[m] / Us.alpha[m];
        if (P.plastic && P.phase[m] == TJ_PHASE_SOLID) Us.are[m] = mult * U.are[m];
        Us.rho += Us.arho[m];
    }
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        if (row == d) Us.rhou[row] = mult * U.rho * Ss;
        else Us.rhou[row] = mult * U.rhou[row];
        Us.vel[row] = Us.rhou[row] / Us.rho;
        if (P.solid)
#pragma unroll
            for (int col = 0; col < 3; ++col)
                Us.V[3 * row + col] = (row == d) ? U.V[3 * row + col] : mult * U.V[3 * row + col];
    }
    Us.E = mult * U.rho * (U.E / U.rho + (Ss - ud) * (Ss - (U.sigma[4 * d]) / (U.rho * (SK - ud))));
}

// Physical flux of the conservative variables (flux.cpp:33-47) into the
// flux-word layout.
__device__ inline void phys_flux(const DevParams& P, const CellS& U, int d, double* F)
{
    double ud = U.vel[d];
    for (int m = 0; m < P.M; ++m) {
        F[P.X_ALPHA + m] = U.alpha[m] * ud;
        F[P.X_ARHO + m] = U.arho[m] * ud;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) F[P.X_RHOU + r] = U.rhou[r] * ud - U.sigma[3 * r + d];
    double vs = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) vs += U.vel[i] * U.sigma[3 * i + d];
    F[P.X_E] = U.E * ud - vs;
    if (P.solid)
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            int row = q / 3, col = q % 3;
            F[P.X_V + q] = U.V[q] * ud - U.V[3 * d + col] * U.vel[row];
        }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) F[P.X_ARE + m] = U.are[m] * ud;
}

// Conservative values of a state in the flux-word layout.
__device__ inline void cons_vals(const DevParams& P, const CellS& U, double* Q)
{
    for (int m = 0; m < P.M; ++m) {
        Q[P.X_ALPHA + m] = U.alpha[m];
        Q[P.X_ARHO + m] = U.arho[m];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) Q[P.X_RHOU + r] = U.rhou[r];
    Q[P.X_E] = U.E;
    if (P.solid)
#pragma unroll
        for (int q = 0; q < 9; ++q) Q[P.X_V + q] = U.V[q];
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) Q[P.X_ARE + m] = U.are[m];
}

#define TJ_MAXX 32

// Returns the side whose star alpha the face carries: 0 left, 1 right.
__device__ inline int face_flux(const DevParams& P, const CellS& L, const CellS& R, int d, double* F, DevScalars* scal)
{
    double x1 = fabs(L.vel[d]) + L.a, x2 = fabs(R.vel[d]) + R.a;
    double SR = (x1 < x2) ? x2 : x1;
    double SL = -SR;
    double Ss = (-R.sigma[4 * d] + L.sigma[4 * d] + L.rhou[d] * (SL - L.vel[d]) - R.rhou[d] * (SR - R.vel[d])) /
                (L.rho * (SL - L.vel[d]) - R.rho * (SR - R.vel[d]));  // getSstar, hllc.cpp:5-8
    F[P.X_SSTAR] = Ss;
    const int nx = P.X_SSTAR;  // words before S*: the conservative variables
    double FK[TJ_MAXX], QK[TJ_MAXX], QS[TJ_MAXX], FS[TJ_MAXX];
    CellS Ls, Rs;
    if (!P.solid) {
        int side;
        const CellS* K;
        double SK;
        bool hllc;
        if (SL >= 0.0) { side = 0; K = &L; SK = SL; hllc = false; }
        else if (Ss >= 0.0) { side = 0; K = &L; SK = SL; hllc = true; }
        else if (SR >= 0.0) { side = 1; K = &R; SK = SR; hllc = true; }
        else { side = 1; K = &R; SK = SR; hllc = false; }
        CellS& Ks = side ? Rs : Ls;
        star_state(P, *K, Ks, SK, Ss, d);
        phys_flux(P, *K, d, FK);
        phys_flux(P, Ks, d, FS);
        cons_vals(P, *K, QK);
        cons_vals(P, Ks, QS);
        for (int w = 0; w < nx; ++w) {
            bool is_alpha = w < P.X_ALPHA + P.M;
            F[w] = is_alpha ? FS[w] : (hllc ? FK[w] + SK * (QS[w] - QK[w]) : FK[w]);
        }
        return side;
    }

    // 5-wave solver for solids (hllc.cpp:133-380).
    if (isnan(SL) || isnan(SR) || isnan(Ss)) { set_status(scal, TJ_ERR_WAVESPEED); return 0; }
    double SLT = 0.0, SRT = 0.0;
    CellS Uss;
    double QL[TJ_MAXX], QR[TJ_MAXX], QLs[TJ_MAXX], QRs[TJ_MAXX], QSS[TJ_MAXX], FL[TJ_MAXX], FR[TJ_MAXX], FAs[TJ_MAXX];
    const double* vsrc;
    int side;
    auto starstar = [&](const CellS& UK, CellS& UKs, double SKT) {  // getStarStarState, hllc.cpp:87-129
        Uss = UKs;
#pragma unroll
        for (int i = 0; i < 3; ++i)  // getSigmaStar, hllc.cpp:75-83
            UKs.sigma[3 * i + d] =
                (Ls.rho * (Ss - SLT) * Rs.rho * (Ss - SRT) * (L.vel[i] - R.vel[i]) + Ls.rho * (Ss - SLT) * R.sigma[3 * i + d] -
                 Rs.rho * (Ss - SRT) * L.sigma[3 * i + d]) /
                (Ls.rho * (Ss - SLT) - Rs.rho * (Ss - SRT));
#pragma unroll
        for (int row = 0; row < 3; ++row) {
            if (row == d) continue;
            Uss.rhou[row] += (UKs.sigma[3 * row + d] - UK.sigma[3 * row + d]) / (Ss - SKT);
            Uss.vel[row] = Uss.rhou[row] / Uss.rho;
        }
#pragma unroll
        for (int row = 0; row < 3; ++row) {
            if (row == d) continue;
            Uss.E += (Uss.vel[row] * UKs.sigma[3 * row + d] - UK.vel[row] * UK.sigma[3 * row + d]) / (Ss - SKT);
#pragma unroll
            for (int col = 0; col < 3; ++col)
                Uss.V[3 * row + col] += (Uss.V[3 * d + col] * (Uss.vel[row] - UK.vel[row])) / (Ss - SKT);
        }
    };
    phys_flux(P, L, d, FL);
    phys_flux(P, R, d, FR);
    cons_vals(P, L, QL);
    cons_vals(P, R, QR);
    if (SL >= 0.0) {
        star_state(P, L, Ls, SL, Ss, d);
        phys_flux(P, Ls, d, FAs);
        for (int w = 0; w < nx; ++w) F[w] = (w < P.X_ALPHA + P.M) ? FAs[w] : FL[w];
        vsrc = L.V;
        side = 0;
    } else if (Ss >= 0.0) {
        star_state(P, L, Ls, SL, Ss, d);
        SLT = Ss - transverse_speed(P, Ls);
        phys_flux(P, Ls, d, FAs);
        cons_vals(P, Ls, QLs);
        if (SLT >= 0.0) {
            for (int w = 0; w < nx; ++w) F[w] = (w < P.X_ALPHA + P.M) ? FAs[w] : FL[w] + SL * (QLs[w] - QL[w]);
            vsrc = Ls.V;
        } else {
            star_state(P, R, Rs, SR, Ss, d);
            SRT = Ss + transverse_speed(P, Rs);
            starstar(L, Ls, SLT);
            cons_vals(P, Uss, QSS);
            for (int w = 0; w < nx; ++w)
                F[w] = (w < P.X_ALPHA + P.M) ? FAs[w] : FL[w] + SL * (QLs[w] - QL[w]) + SLT * (QSS[w] - QLs[w]);
            vsrc = Uss.V;
        }
        side = 0;
    } else if (SR >= 0.0) {
        star_state(P, R, Rs, SR, Ss, d);
        SRT = Ss + transverse_speed(P, Rs);
        phys_flux(P, Rs, d, FAs);
        cons_vals(P, Rs, QRs);
        if (SRT >= 0.0) {
            star_state(P, L, Ls, SL, Ss, d);
            SLT = Ss - transverse_speed(P, Ls);
            starstar(R, Rs, SRT);
            cons_vals(P, Uss, QSS);
            for (int w = 0; w < nx; ++w)
                F[w] = (w < P.X_ALPHA + P.M) ? FAs[w] : FR[w] + SR * (QRs[w] - QR[w]) + SRT * (QSS[w] - QRs[w]);
            vsrc = Uss.V;
        } else {
            for (int w = 0; w < nx; ++w) F[w] = (w < P.X_ALPHA + P.M) ? FAs[w] : FR[w] + SR * (QRs[w] - QR[w]);
            vsrc = Rs.V;
        }
        side = 1;
    } else {
        star_state(P, R, Rs, SR, Ss, d);
        phys_flux(P, Rs, d, FAs);
        for (int w = 0; w < nx; ++w) F[w] = (w < P.X_ALPHA + P.M) ? FAs[w] : FR[w];
        vsrc = R.V;
        side = 1;
    }
#pragma unroll
    for (int col = 0; col < 3; ++col) F[P.X_VSTAR + col] = vsrc[3 * d + col];  // VSTAR(d, col), read by update
    if (isnan(SL) || isnan(SR) || isnan(Ss) || isnan(SLT) || isnan(SRT)) set_status(scal, TJ_ERR_WAVESPEED);
    return side;
}

__global__ void k_flux(DevParams P, Fp64Bufs b, int d)
{
    if (b.scal->done) return;
    const long long nt = b.ntot, nf = b.nftot[d];
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x) {
        const int q = find_dom_face(b.doms, b.ndom, d, f);
        const DevDomain D = b.doms[q];
        int nfv[3] = {D.n[0], D.n[1], D.n[2]};
        nfv[d] += 1;
        long long l = f - D.foff[d];
        int i = (int)(l % nfv[0]), j = (int)((l / nfv[0]) % nfv[1]), k = (int)(l / ((long long)nfv[0] * nfv[1]));
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int rl[3], rr[3];
        long long gl = map_cell(P, D, i - o[0], j - o[1], k - o[2], rl);
        long long gr = map_cell(P, D, i, j, k, rr);
        CellS L, R;
        load_face(P, b.UR, nt, gl, rl[d] ? d : -1, L);
        load_face(P, b.UL, nt, gr, rr[d] ? d : -1, R);
        double F[TJ_MAXX];
        int side = face_flux(P, L, R, d, F, b.scal);
        for (int w = 0; w < P.NX; ++w) b.FX[(long long)w * nf + f] = F[w];
        if (P.thinc) {
            const CellS& src = side ? R : L;
            int idx[3] = {i, j, k};
            if (idx[d] < D.n[d]) {  // ULStar alpha at the valid cell of this face
                long long g = D.off + i + (long long)D.n[0] * (j + (long long)D.n[1] * k);
                for (int m = 0; m < P.M; ++m) b.ulstar[(long long)m * nt + g] = src.alpha[m];
            }
            if (idx[d] >= 1) {  // the ghost hi+1 of the box to the left, if this is its hi face
                long long gL = D.off + (i - o[0]) + (long long)D.n[0] * ((j - o[1]) + (long long)D.n[1] * (k - o[2]));
                const int* bx = b.boxes + 6 * (D.box_off + b.cell_box[gL]);
                if (bx[3 + d] == idx[d] - 1)
                    for (int m = 0; m < P.M; ++m) b.gstar[d][(long long)m * nf + f] = src.alpha[m];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Plastic radial return (plastic.cpp:83-223) and cleanUpV (:476-528).
// ---------------------------------------------------------------------------
__device__ inline int plastic_cell(const DevParams& P, CellS& c)
{
    double tsolid = 0.0;
    for (int m = 0; m < P.M; ++m)
        if (P.phase[m] == TJ_PHASE_SOLID) tsolid += c.alpha[m];
    if (tsolid <= 0.5) {  // cellIsMostlyFluid
        for (int m = 0; m < P.M; ++m) { c.eps[m] = 0.0; c.are[m] = 0.0; }
        return 0;
    }
    hencky(P, c);
    double JT = 0.0, JB = 0.0, norm = 0.0, J, Jn;
    for (int m = 0; m < P.M; ++m) {
        ECell e = ecell_of(c, m);
        if (P.phase[m] == TJ_PHASE_SOLID) {
            J = sqrt(c.hj2);
            double G = eos_G(P, m, e);
            if (G * J * sqrt(3.0) > P.yield[m]) Jn = P.yield[m] / (sqrt(3.0) * G);
            else Jn = J;
            c.eps[m] += sqrt(2.0 / 3.0) * (J - Jn);
            c.are[m] = c.eps[m] * c.arho[m];
        } else {
            J = 0.0;
            Jn = 0.0;
            c.eps[m] = 0.0;
            c.are[m] = 0.0;
        }
        JB += (eos_invG(P, m, e)) * J;
        JT += (eos_invG(P, m, e)) * Jn;
        norm += (eos_invG(P, m, e));
    }
    JB *= 1.0 / norm;
    JT *= 1.0 / norm;
    if (JB == 0.0 && JT == 0.0) { JB = 1.0; JT = 1.0; }
    double t1[9], t2[9], t2i[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            double& dv = c.devH[3 * r + q];
            if (dv != 0.0 && JB == 0.0 && JT != 0.0) return TJ_ERR_PLASTIC;
            dv *= JT / JB;
            t1[3 * r + q] = (double)(r == q) + 0.5 * dv;
            t2[3 * r + q] = (double)(r == q) - 0.5 * dv;
        }
    invert3(t2, t2i);
    mm3(t2i, t1, c.V);
    return 0;
}

__device__ inline void cleanup_v_cell(const DevParams& P, CellS& c)
{
    double ta = 0.0, ts = 0.0;
    for (int m = 0; m < P.M; ++m) {
        ta += c.alpha[m];
        if (P.phase[m] == TJ_PHASE_SOLID) ts += c.alpha[m];
    }
    double B[9], Sq[9];
    mmT3(c.V, c.V, B);
    sqrtm3(B, Sq);
    double norm = tjm_pow(det3(Sq), -1.0 / 3.0);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) c.V[3 * r + q] = ((Sq[3 * r + q] * norm * ts) + (double)(r == q) * (ta - ts)) / ta;
}

// contains_nan over the conservative and primitive lists of one cell.
__device__ inline bool cell_has_nan(const DevParams& P, const CellS& c)
{
    bool n = false;
    for (int m = 0; m < P.M; ++m) n |= isnan(c.alpha[m]) || isnan(c.arho[m]) || isnan(c.rhok[m]);
#pragma unroll
    for (int r = 0; r < 3; ++r) n |= isnan(c.rhou[r]) || isnan(c.vel[r]);
    n |= isnan(c.E) || isnan(c.p);
    if (P.solid)
#pragma unroll
        for (int q = 0; q < 9; ++q) n |= isnan(c.V[q]);
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) n |= isnan(c.eps[m]) || isnan(c.are[m]);
    return n;
}

// ---------------------------------------------------------------------------
// Update of one direction; last direction: c2p; second stage: average and
// the post-advance operators of main.cpp:145-187.
// ---------------------------------------------------------------------------
__global__ void k_update(DevParams P, Fp64Bufs b, const double* __restrict__ X, double* Y, int d, int first, int last,
                         int finish)
{
    if (b.scal->done) return;
    const long long nt = b.ntot, nf = b.nftot[d];
    const double dtdx_num = b.scal->dt;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        const int q = find_dom(b.doms, b.ndom, g);
        const DevDomain D = b.doms[q];
        long long l = g - D.off;
        int i = (int)(l % D.n[0]), j = (int)((l / D.n[0]) % D.n[1]), k = (int)(l / ((long long)D.n[0] * D.n[1]));
        int o[3] = {0, 0, 0};
        o[d] = 1;
        const long long f0 = face_index(D, d, i, j, k), f1 = face_index(D, d, i + o[0], j + o[1], k + o[2]);
        CellS U, Yc;
        load_state(P, X, nt, g, nullptr, U);
        if (first) Yc = U;
        else load_state(P, Y, nt, g, nullptr, Yc);
        const double dtdx = dtdx_num / D.dx[d];
#define FXW(w, f) b.FX[(long long)(w)*nf + (f)]
        const double dS = FXW(P.X_SSTAR, f0) - FXW(P.X_SSTAR, f1);
        for (int m = 0; m < P.M; ++m) {
            Yc.alpha[m] += dtdx * (FXW(P.X_ALPHA + m, f0) - FXW(P.X_ALPHA + m, f1) - U.alpha[m] * (FXW(P.X_SSTAR, f0) - FXW(P.X_SSTAR, f1)));
            Yc.arho[m] += dtdx * (FXW(P.X_ARHO + m, f0) - FXW(P.X_ARHO + m, f1));
        }
        (void)dS;
#pragma unroll
        for (int r = 0; r < 3; ++r) Yc.rhou[r] += dtdx * (FXW(P.X_RHOU + r, f0) - FXW(P.X_RHOU + r, f1));
        Yc.E += dtdx * (FXW(P.X_E, f0) - FXW(P.X_E, f1));
        if (P.solid)
#pragma unroll
            for (int qq = 0; qq < 9; ++qq) {
                int row = qq / 3, col = qq % 3;
                Yc.V[qq] += dtdx * (FXW(P.X_V + qq, f0) - FXW(P.X_V + qq, f1) -
                                    (2.0 / 3.0) * U.V[qq] * (FXW(P.X_SSTAR, f0) - FXW(P.X_SSTAR, f1)) +
                                    U.vel[row] * (FXW(P.X_VSTAR + col, f0) - FXW(P.X_VSTAR + col, f1)));
            }
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) Yc.are[m] += dtdx * (FXW(P.X_ARE + m, f0) - FXW(P.X_ARE + m, f1));
#undef FXW
        if (last) {
            c2p(P, Yc);
            if (finish) {
                // U1 = U*0.5 + U2*0.5 over every carried component (hllc.cpp:705)
                CellS A0;
                load_state(P, b.A, nt, g, nullptr, A0);
                for (int m = 0; m < P.M; ++m) {
                    Yc.alpha[m] = (A0.alpha[m] * (1.0 / 2.0)) + (Yc.alpha[m] * (1.0 / 2.0));
                    Yc.arho[m] = (A0.arho[m] * (1.0 / 2.0)) + (Yc.arho[m] * (1.0 / 2.0));
                    Yc.rhok[m] = (A0.rhok[m] * (1.0 / 2.0)) + (Yc.rhok[m] * (1.0 / 2.0));
                    if (P.plastic) {
                        Yc.eps[m] = (A0.eps[m] * (1.0 / 2.0)) + (Yc.eps[m] * (1.0 / 2.0));
                        Yc.are[m] = (A0.are[m] * (1.0 / 2.0)) + (Yc.are[m] * (1.0 / 2.0));
                    }
                }
                Yc.rho = (A0.rho * (1.0 / 2.0)) + (Yc.rho * (1.0 / 2.0));
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    Yc.rhou[r] = (A0.rhou[r] * (1.0 / 2.0)) + (Yc.rhou[r] * (1.0 / 2.0));
                    Yc.vel[r] = (A0.vel[r] * (1.0 / 2.0)) + (Yc.vel[r] * (1.0 / 2.0));
                }
                Yc.E = (A0.E * (1.0 / 2.0)) + (Yc.E * (1.0 / 2.0));
                Yc.p = (A0.p * (1.0 / 2.0)) + (Yc.p * (1.0 / 2.0));
                if (P.solid) {
#pragma unroll
                    for (int qq = 0; qq < 9; ++qq) Yc.V[qq] = (A0.V[qq] * (1.0 / 2.0)) + (Yc.V[qq] * (1.0 / 2.0));
                    Yc.hj2 = (A0.hj2 * (1.0 / 2.0)) + (Yc.hj2 * (1.0 / 2.0));
                }
                if (finish == 2) {  // advance() alone: the average only
                    store_state(P, b.A, nt, g, Yc);
                    continue;
                }
                if (P.plastic) {
                    int e = plastic_cell(P, Yc);
                    if (e) set_status(b.scal, e);
                    c2p(P, Yc);
                }
                if (P.solid) cleanup_v_cell(P, Yc);
                int e = cleanup_alpha(P, Yc.alpha);
                if (e) set_status(b.scal, e);
                if (b.cell_box[g] == D.nbox - 1 && cell_has_nan(P, Yc)) atomicOr(&b.scal->nan_flag, 1);
                store_state(P, b.A, nt, g, Yc);
                continue;
            }
        }
        store_state(P, Y, nt, g, Yc);
    }
}

// ---------------------------------------------------------------------------
// CFL (timestep.cpp:7-70) and device-side time bookkeeping (main.cpp:121-143).
// ---------------------------------------------------------------------------
__global__ void k_cfl(DevParams P, Fp64Bufs b, const double* __restrict__ X)
{
    if (b.scal->done) return;
    const long long nt = b.ntot;
    double mn = 1.79769313486231570815e+308;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        const int q = find_dom(b.doms, b.ndom, g);
        const DevDomain D = b.doms[q];
        CellS c;
        load_state(P, X, nt, g, nullptr, c);
        double a = sound_speed(P, c);
        for (int n = 0; n < P.dim; ++n) {
            double v = D.dx[n] / (a + fabs(c.vel[n]));
            if (v < mn) mn = v;
        }
    }
    for (int s = 16; s > 0; s >>= 1) {
        double o = __shfl_down_sync(0xffffffffu, mn, s);
        if (o < mn) mn = o;
    }
    __shared__ double red[32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) red[w] = mn;
    __syncthreads();
    if (w == 0) {
        mn = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 1.79769313486231570815e+308;
        for (int s = 16; s > 0; s >>= 1) {
            double o = __shfl_down_sync(0xffffffffu, mn, s);
            if (o < mn) mn = o;
        }
        if (lane == 0) atomicMin(&b.scal->dtmin_bits, (unsigned long long)__double_as_longlong(mn));
    }
}

__global__ void k_dt_finalize(DevParams P, DevScalars* s, int clamp)
{
    if (threadIdx.x != 0) return;
    double raw = __longlong_as_double((long long)s->dtmin_bits);
    s->dtmin_raw = raw;
    s->dtmin_bits = 0x7FEFFFFFFFFFFFFFull;
    if (!clamp) return;
    if (s->done) return;
    if (!(s->t < s->t_end)) { s->done = 1; return; }
    double dt = P.cfl * raw;
    if (s->t + dt > s->t_end) dt = s->t_end - s->t;
    if (s->n < 5) dt *= 0.2;
    s->dt = dt;
}

__global__ void k_step_end(DevScalars* s)
{
    if (threadIdx.x != 0 || s->done) return;
    if (s->nan_flag) {
        s->done = 1;
        atomicCAS(&s->status, 0, TJ_ERR_NAN);
        return;
    }
    s->t += s->dt;
    s->n += 1;
}

__global__ void k_set_dt(DevScalars* s, double dt)
{
    if (threadIdx.x != 0) return;
    s->dt = dt;
    s->done = 0;
}

// ---------------------------------------------------------------------------
// Whole-array cell operators of the C ABI.
// ---------------------------------------------------------------------------
__global__ void k_cell_op(DevParams P, Fp64Bufs b, double* X, const double* X2, int op)
{
    const long long nt = b.ntot;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        CellS c;
        load_state(P, X, nt, g, nullptr, c);
        if (P.solid && (op == OP_P2C)) {
            // the primitive list carries V; HJ2 recomputed by p2c
        }
        switch (op) {
            case OP_C2P: c2p(P, c); break;
            case OP_P2C: p2c(P, c); break;
            case OP_CLEAN_ALPHA: {
                int e = cleanup_alpha(P, c.alpha);
                if (e) set_status(b.scal, e);
                break;
            }
            case OP_CLEAN_V: cleanup_v_cell(P, c); break;
            case OP_PLASTIC: {
                int e = plastic_cell(P, c);
                if (e) set_status(b.scal, e);
                c2p(P, c);
                break;
            }
            case OP_NAN: {
                const int q = find_dom(b.doms, b.ndom, g);
                if (b.cell_box[g] == b.doms[q].nbox - 1 && cell_has_nan(P, c)) atomicOr(&b.scal->nan_flag, 1);
                continue;
            }
            default: break;
        }
        store_state(P, X, nt, g, c);
    }
}

// AccessPattern blocks <-> carried state, for one box of one domain. The AP
// array is indexed ap[n*cstride + (i+go) + ld_i*((j+go) + ld_j*(k+go))] for box
// cell (i,j,k) relative to the box lo, where go is the ghost offset.
__global__ void k_ap_to_state(DevParams P, Fp64Bufs b, int dom, int lx, int ly, int lz, int nx, int ny, int nz,
                              const double* ap, int ld_i, int ld_j, long long cs, int go, double* X)
{
    const long long nt = b.ntot, nb = (long long)nx * ny * nz;
    const DevDomain D = b.doms[dom];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nb; t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / ((long long)nx * ny));
        long long src = (i + go) + (long long)ld_i * ((j + (P.dim > 1 ? go : 0)) + (long long)ld_j * (k + (P.dim > 2 ? go : 0)));
        long long g = D.off + (lx + i) + (long long)D.n[0] * ((ly + j) + (long long)D.n[1] * (lz + k));
#define APV(comp) ap[(long long)(comp)*cs + src]
        for (int m = 0; m < P.M; ++m) {
            X[(P.S_ALPHA + m) * nt + g] = APV(P.A_ALPHA + m);
            X[(P.S_ARHO + m) * nt + g] = APV(P.A_ARHO + m);
            X[(P.S_RHOK + m) * nt + g] = APV(P.A_RHOK + m);
        }
        X[P.S_RHO * nt + g] = APV(P.A_RHO);
        for (int r = 0; r < 3; ++r) {
            X[(P.S_RHOU + r) * nt + g] = APV(P.A_RHOU + r);
            X[(P.S_VEL + r) * nt + g] = APV(P.A_VEL + r);
        }
        X[P.S_E * nt + g] = APV(P.A_E);
        X[P.S_P * nt + g] = APV(P.A_P);
        if (P.solid) {
            for (int qq = 0; qq < 9; ++qq) X[(P.S_V + qq) * nt + g] = APV(P.A_V + qq);
            X[P.S_HJ2 * nt + g] = APV(P.A_HJ2);
        }
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) {
                X[(P.S_EPS + m) * nt + g] = APV(P.A_EPS + m);
                X[(P.S_ARE + m) * nt + g] = APV(P.A_ARE + m);
            }
#undef APV
    }
}

__global__ void k_state_to_ap(DevParams P, Fp64Bufs b, int dom, int lx, int ly, int lz, int nx, int ny, int nz,
                              const double* X, double* ap, int ld_i, int ld_j, long long cs, int go)
{
    const long long nt = b.ntot, nb = (long long)nx * ny * nz;
    const DevDomain D = b.doms[dom];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nb; t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / ((long long)nx * ny));
        long long dst = (i + go) + (long long)ld_i * ((j + (P.dim > 1 ? go : 0)) + (long long)ld_j * (k + (P.dim > 2 ? go : 0)));
        long long g = D.off + (lx + i) + (long long)D.n[0] * ((ly + j) + (long long)D.n[1] * (lz + k));
        CellS c;
        load_state(P, X, nt, g, nullptr, c);
        // Derived components: Hencky strain and stress of the carried state,
        // sound speed; USTAR / VSTAR are scratch in the reference.
        double hj2 = c.hj2;
        if (P.solid) hencky(P, c);
        if (P.solid) c.hj2 = hj2;
        stress(P, c);
        c.a = sound_speed(P, c);
#define APV(comp) ap[(long long)(comp)*cs + dst]
        for (int m = 0; m < P.M; ++m) {
            APV(P.A_ALPHA + m) = c.alpha[m];
            APV(P.A_ARHO + m) = c.arho[m];
            APV(P.A_RHOK + m) = c.rhok[m];
        }
        APV(P.A_RHO) = c.rho;
        for (int r = 0; r < 3; ++r) {
            APV(P.A_RHOU + r) = c.rhou[r];
            APV(P.A_VEL + r) = c.vel[r];
        }
        APV(P.A_E) = c.E;
        APV(P.A_P) = c.p;
        APV(P.A_A) = c.a;
        APV(P.A_USTAR) = 0.0;
        for (int qq = 0; qq < 9; ++qq) APV(P.A_SIGMA + qq) = c.sigma[qq];
        if (P.solid) {
            for (int qq = 0; qq < 9; ++qq) {
                APV(P.A_V + qq) = c.V[qq];
                APV(P.A_VSTAR + qq) = 0.0;
                APV(P.A_DEVH + qq) = c.devH[qq];
            }
            APV(P.A_HJ2) = c.hj2;
        }
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) {
                APV(P.A_EPS + m) = c.eps[m];
                APV(P.A_ARE + m) = c.are[m];
            }
#undef APV
    }
}

__global__ void k_prim_to_state(DevParams P, Fp64Bufs b, int dom, const double* prim, double* X)
{
    const long long nt = b.ntot;
    const DevDomain D = b.doms[dom];
    const long long nd = (long long)D.n[0] * D.n[1] * D.n[2];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nd; t += (long long)gridDim.x * blockDim.x) {
        CellS c;
        int w = 0;
        for (int m = 0; m < P.M; ++m) c.alpha[m] = prim[(w++) * nd + t];
        for (int m = 0; m < P.M; ++m) c.rhok[m] = prim[(w++) * nd + t];
        for (int r = 0; r < 3; ++r) c.vel[r] = prim[(w++) * nd + t];
        c.p = prim[(w++) * nd + t];
        c.hj2 = 0.0;
        if (P.solid)
            for (int qq = 0; qq < 9; ++qq) c.V[qq] = prim[(w++) * nd + t];
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) c.eps[m] = prim[(w++) * nd + t];
        p2c(P, c);
        store_state(P, X, nt, D.off + t, c);
    }
}

// ---------------------------------------------------------------------------
// Host launchers.
// ---------------------------------------------------------------------------
#define PROF_BEGIN(name) \
    if (pr) pr->begin(name, st)
#define PROF_END(name) \
    if (pr) pr->end(name, st)

int fp64_cfl(const DevParams& P, const Fp64Bufs& b, const double* X, cudaStream_t st, Prof* pr)
{
    PROF_BEGIN("tj_cfl_fp64");
    k_cfl<<<nblocks(b.ntot), kThreads, 0, st>>>(P, b, X);
    PROF_END("tj_cfl_fp64");
    return 1;
}

int fp64_dt_finalize(const DevParams& P, const Fp64Bufs& b, int clamp, cudaStream_t st)
{
    k_dt_finalize<<<1, 32, 0, st>>>(P, b.scal, clamp);
    return 1;
}

int fp64_stage(const DevParams& P, const Fp64Bufs& b, const double* X, double* Y, int finish, cudaStream_t st, Prof* pr)
{
    int n = 0;
    for (int d = 0; d < P.dim; ++d) {
        PROF_BEGIN("tj_recon_fp64");
        k_recon<<<nblocks(b.ntot), kThreads, 0, st>>>(P, b, X, d);
        PROF_END("tj_recon_fp64");
        PROF_BEGIN("tj_flux_fp64");
        k_flux<<<nblocks(b.nftot[d]), kThreads, 0, st>>>(P, b, d);
        PROF_END("tj_flux_fp64");
        PROF_BEGIN("tj_update_fp64");
        k_update<<<nblocks(b.ntot), kThreads, 0, st>>>(P, b, X, Y, d, d == 0, d == P.dim - 1, finish);
        PROF_END("tj_update_fp64");
        n += 3;
    }
    return n;
}

int fp64_step_end(const Fp64Bufs& b, cudaStream_t st)
{
    k_step_end<<<1, 32, 0, st>>>(b.scal);
    return 1;
}

int fp64_set_dt(const Fp64Bufs& b, double dt, cudaStream_t st)
{
    k_set_dt<<<1, 32, 0, st>>>(b.scal, dt);
    return 1;
}

int fp64_cell_op(const DevParams& P, const Fp64Bufs& b, double* X, const double* X2, int op, cudaStream_t st)
{
    k_cell_op<<<nblocks(b.ntot), kThreads, 0, st>>>(P, b, X, X2, op);
    return 1;
}

int fp64_ap_to_state(const DevParams& P, const Fp64Bufs& b, int dom, const int* bx, const double* ap, int ld_i, int ld_j,
                     int ld_k, long long cs, int go, double* X, cudaStream_t st)
{
    (void)ld_k;
    int nx = bx[3] - bx[0] + 1, ny = bx[4] - bx[1] + 1, nz = bx[5] - bx[2] + 1;
    k_ap_to_state<<<nblocks((long long)nx * ny * nz), kThreads, 0, st>>>(P, b, dom, bx[0], bx[1], bx[2], nx, ny, nz, ap, ld_i,
                                                                         ld_j, cs, go, X);
    return 1;
}

int fp64_state_to_ap(const DevParams& P, const Fp64Bufs& b, int dom, const int* bx, const double* X, double* ap, int ld_i,
                     int ld_j, int ld_k, long long cs, int go, cudaStream_t st)
{
    (void)ld_k;
    int nx = bx[3] - bx[0] + 1, ny = bx[4] - bx[1] + 1, nz = bx[5] - bx[2] + 1;
    k_state_to_ap<<<nblocks((long long)nx * ny * nz), kThreads, 0, st>>>(P, b, dom, bx[0], bx[1], bx[2], nx, ny, nz, X, ap,
                                                                         ld_i, ld_j, cs, go);
    return 1;
}

int fp64_prim_to_state(const DevParams& P, const Fp64Bufs& b, int dom, const double* prim, double* X, cudaStream_t st)
{
    k_prim_to_state<<<nblocks(b.ntot), kThreads, 0, st>>>(P, b, dom, prim, X);
    return 1;
}

}  // namespace tj
