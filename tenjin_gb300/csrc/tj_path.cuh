// The per-direction kernels of the per-timestep update (reconstruction, face
// flux, update), one source for two working types: PT = DevParams (binary64,
// the reference's evaluation order: bit-exact parity, compiled with
// -fmad=false in tj_fp64.cu) and PT = DevParams32 (binary32 bulk, tj_fp32.cu).
// The binary32 instance keeps the total energy as a compensated pair (E, Elo),
// closes the pressure in binary64 (in c2p) and runs the plastic return map in
// binary64 (plastic_cell_proj64); everything else is the same code.
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
#pragma once

#include <cuda_runtime.h>

#include "tj_device.cuh"
#include "tj_fp64.cuh"

namespace tj {

// Error-free accumulation of b into the pair (hi, lo) (binary32 energy).
__device__ __forceinline__ void dd_add32(float& hi, float& lo, float b)
{
    const float s = __fadd_rn(hi, b);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    lo = __fadd_rn(lo, e);
    const float t = __fadd_rn(s, lo);
    lo = __fsub_rn(lo, __fsub_rn(t, s));
    hi = t;
}

// (ah + al) / 2 + (bh + bl) / 2 into (bh, bl) (the RK2 average of the energy).
__device__ __forceinline__ void avg_pair32(float ah, float al, float& bh, float& bl)
{
    float hs = 0.5f * ah, ls = 0.5f * al;
    dd_add32(hs, ls, 0.5f * bh);
    ls = __fadd_rn(ls, 0.5f * bl);
    const float t = __fadd_rn(hs, ls);
    bl = __fsub_rn(ls, __fsub_rn(t, hs));
    bh = t;
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

// (i, j, k) of entry l of an n0 x n1 x n2 block (i fastest). One domain's
// cells and faces number below 2^32 at any size that fits the device, so the
// division runs in 32-bit unsigned arithmetic (a 64-bit division is a long
// software sequence); the 64-bit form remains for larger blocks.
__device__ __forceinline__ void split3(long long l, int n0, int n1, int& i, int& j, int& k)
{
    if ((unsigned long long)l < 4294967296ULL) {
        const unsigned u = (unsigned)l, q = u / (unsigned)n0;
        i = (int)(u - q * (unsigned)n0);
        const unsigned k2 = q / (unsigned)n1;
        j = (int)(q - k2 * (unsigned)n1);
        k = (int)k2;
    } else {
        i = (int)(l % n0);
        j = (int)((l / n0) % n1);
        k = (int)(l / ((long long)n0 * n1));
    }
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
template <typename PT, typename R = typename PT::real>
__device__ __forceinline__ long long map_cell(const PT& P, const DevDomain& D, int i, int j, int k, int* refl)
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
template <typename PT, typename R = typename PT::real>
__device__ inline void load_state(const PT& P, const R* X, long long nt, long long g, const int* refl,
                                  CellT<R>& c)
{
    for (int m = 0; m < P.M; ++m) {
        c.alpha[m] = X[(P.S_ALPHA + m) * nt + g];
        c.arho[m] = X[(P.S_ARHO + m) * nt + g];
        c.rhok[m] = X[(P.S_RHOK + m) * nt + g];
    }
    c.rho = X[P.S_RHO * nt + g];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        R u = X[(P.S_VEL + r) * nt + g], ru = X[(P.S_RHOU + r) * nt + g];
        if (refl && refl[r]) { u = -u; ru = -ru; }
        c.vel[r] = u;
        c.rhou[r] = ru;
    }
    c.E = X[P.S_E * nt + g];
    if constexpr (sizeof(R) == 4) c.Elo = X[P.S_ELO * nt + g];
    c.p = X[P.S_P * nt + g];
    c.hj2 = R(0.0);
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
    if (P.nmix) {
        c.rm0 = X[P.S_RMIX * nt + g];
        c.rm1 = X[(P.S_RMIX + 1) * nt + g];
        c.lam = X[P.S_LAM * nt + g];
        c.arl = X[P.S_ARL * nt + g];
    }
}

// The fields of a carried cell that reconstruction reads (load_state without
// the conservative variables, which primitiveToConservative recomputes on
// each face state): the primitives with the reflect_odd sign, the cell's own
// HJ2 (SOLID) and alphaRhoEps (PLASTIC), and lambda (mixtures).
template <typename PT, typename R = typename PT::real>
__device__ inline void load_prims(const PT& P, const R* X, long long nt, long long g, const int* refl, CellT<R>& c)
{
    for (int m = 0; m < P.M; ++m) {
        c.alpha[m] = X[(P.S_ALPHA + m) * nt + g];
        c.rhok[m] = X[(P.S_RHOK + m) * nt + g];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        R u = X[(P.S_VEL + r) * nt + g];
        if (refl && refl[r]) u = -u;
        c.vel[r] = u;
    }
    c.p = X[P.S_P * nt + g];
    c.hj2 = R(0.0);
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
    if (P.nmix) c.lam = X[P.S_LAM * nt + g];
}

template <typename PT, typename R = typename PT::real>
__device__ inline void store_state(const PT& P, R* X, long long nt, long long g, const CellT<R>& c)
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
    if constexpr (sizeof(R) == 4) X[P.S_ELO * nt + g] = c.Elo;
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
    if (P.nmix) {
        X[P.S_RMIX * nt + g] = c.rm0;
        X[(P.S_RMIX + 1) * nt + g] = c.rm1;
        X[P.S_LAM * nt + g] = c.lam;
        X[P.S_ARL * nt + g] = c.arl;
    }
}

template <typename PT, typename R = typename PT::real>
__device__ inline void store_face(const PT& P, R* F, long long nt, long long g, const CellT<R>& c)
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
    if (P.nmix) F[P.F_ARL * nt + g] = c.arl;
}

template <typename PT, typename R = typename PT::real>
__device__ inline void load_face(const PT& P, const R* F, long long nt, long long g, int oddir, CellT<R>& c)
{
    for (int m = 0; m < P.M; ++m) {
        c.alpha[m] = F[(P.F_ALPHA + m) * nt + g];
        c.arho[m] = F[(P.F_ARHO + m) * nt + g];
        c.rhok[m] = R(0.0);
    }
    c.rho = F[P.F_RHO * nt + g];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        R u = F[(P.F_VEL + r) * nt + g], ru = F[(P.F_RHOU + r) * nt + g];
        if (r == oddir) { u = -u; ru = -ru; }
        c.vel[r] = u;
        c.rhou[r] = ru;
    }
    c.E = F[P.F_E * nt + g];
    c.p = F[P.F_P * nt + g];
    c.a = F[P.F_A * nt + g];
    c.hj2 = R(0.0);
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
            for (int q = 0; q < 3; ++q) c.sigma[3 * r + q] = -c.p * (R)(r == q);  // stressTensor, fluid
    }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) c.are[m] = F[(P.F_ARE + m) * nt + g];
    if (P.nmix) c.arl = F[P.F_ARL * nt + g];
}

// Without BVD-THINC (whose repeated cleanUpAlpha feeds the closures one
// alpha and the flux another) and without mixtures, the reconstruction
// stores the primitives of each face state -- alpha[M], rho_k[M], u[3], p,
// V[9] (solids), epsilon[M] (plastic): 16 words for the copper plate instead
// of the 31 of a closed state -- and the flux kernel closes them
// (primitiveToConservative, getSoundSpeed) where it reads them: the same
// calls on the same values, so the same bits reach the Riemann solver.
template <typename PT>
__device__ __forceinline__ bool compact_faces(const PT& P)
{
    return !P.thinc && !P.nmix;
}

template <typename PT, typename R = typename PT::real>
__device__ inline void store_prim_face(const PT& P, R* F, long long nt, long long g, const CellT<R>& c)
{
    int w = 0;
    for (int m = 0; m < P.M; ++m) F[(long long)(w++) * nt + g] = c.alpha[m];
    for (int m = 0; m < P.M; ++m) F[(long long)(w++) * nt + g] = c.rhok[m];
#pragma unroll
    for (int r = 0; r < 3; ++r) F[(long long)(w++) * nt + g] = c.vel[r];
    F[(long long)(w++) * nt + g] = c.p;
    if (P.solid) {
#pragma unroll
        for (int q = 0; q < 9; ++q) F[(long long)(w++) * nt + g] = c.V[q];
        if (!P.any_solid) F[(long long)(w++) * nt + g] = c.hj2;  // getHenckyJ2 does not run: the cell's own
    }
    if (P.plastic)  // epsilon of a solid closes alphaRhoEps; a fluid's alphaRhoEps is the cell's own
        for (int m = 0; m < P.M; ++m) F[(long long)(w++) * nt + g] = P.phase[m] == TJ_PHASE_SOLID ? c.eps[m] : c.are[m];
}

// The closed face state of load_face from stored primitives: the closures
// of the reconstruction, then the fields load_face leaves at zero, then the
// reflect_odd sign of a boundary image.
template <typename PT, typename R = typename PT::real>
__device__ inline void load_prim_face(const PT& P, const R* F, long long nt, long long g, int oddir, CellT<R>& c)
{
    int w = 0;
    for (int m = 0; m < P.M; ++m) c.alpha[m] = F[(long long)(w++) * nt + g];
    for (int m = 0; m < P.M; ++m) c.rhok[m] = F[(long long)(w++) * nt + g];
#pragma unroll
    for (int r = 0; r < 3; ++r) c.vel[r] = F[(long long)(w++) * nt + g];
    c.p = F[(long long)(w++) * nt + g];
    c.hj2 = R(0.0);
    if (P.solid) {
#pragma unroll
        for (int q = 0; q < 9; ++q) c.V[q] = F[(long long)(w++) * nt + g];
        if (!P.any_solid) c.hj2 = F[(long long)(w++) * nt + g];
    }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) {
            const R v = F[(long long)(w++) * nt + g];
            if (P.phase[m] == TJ_PHASE_SOLID) c.eps[m] = v;
            else c.are[m] = v;
        }
    p2c(P, c);
    c.a = sound_speed(P, c);
    for (int m = 0; m < P.M; ++m) c.rhok[m] = R(0.0);
    c.hj2 = R(0.0);
    if (!P.solid)
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int q = 0; q < 3; ++q) c.sigma[3 * r + q] = -c.p * (R)(r == q);  // stressTensor, fluid
    if (oddir >= 0) {
        c.vel[oddir] = -c.vel[oddir];
        c.rhou[oddir] = -c.rhou[oddir];
    }
}

template <typename R>
__device__ __forceinline__ R vanleer(R r)  // hllc.cpp:527-537
{
    if (r <= R(0.0)) return R(0.0);
    R a = R(2.0) / (R(1.0) + r), b = R(2.0) * r / (R(1.0) + r);
    return (b < a) ? b : a;
}

template <typename R>
__device__ __forceinline__ void muscl1(R um, R u0, R up, R& l, R& r)  // hllc.cpp:557-568
{
    R rr = (u0 - um) / (up - u0);
    if (isinf(rr) || isnan(rr)) rr = R(0.0);
    R grad = vanleer(rr) * R(0.5) * (up - um);
    l = u0 - R(0.5) * grad;
    r = u0 + R(0.5) * grad;
}

// One carried word at a possibly-ghost cell.
template <typename PT, typename R = typename PT::real>
__device__ __forceinline__ R gv(const PT& P, const DevDomain& D, const R* X, long long nt, int word,
                                     int i, int j, int k)
{
    int refl[3];
    long long g = map_cell(P, D, i, j, k, refl);
    R v = X[word * nt + g];
    for (int d = 0; d < P.dim; ++d)
        if (refl[d] && (word == P.S_VEL + d || word == P.S_RHOU + d)) v = -v;
    return v;
}

// ---------------------------------------------------------------------------
// BVD-THINC candidate of one cell (thinc.cpp:67-147).
// ---------------------------------------------------------------------------
template <typename R>
struct ThincCand {
    int mixed[TJ_MAX_MAT];
    R L[TJ_MAX_MAT], Rv[TJ_MAX_MAT];
    int flag;
};

template <typename PT, typename R = typename PT::real>
__device__ inline R youngs(const PT& P, const DevDomain& D, const R* X, long long nt, int m, int i,
                                int j, int k, int d)  // thinc.cpp:28-53
{
    int a = P.S_ALPHA + m;
#define NB(di, dj) gv(P, D, X, nt, a, i + (di), j + (dj), k)
    R nx = -R(1.0) / (R(8.0) * (R)D.dx[0]) * (NB(1, 1) + R(2.0) * NB(1, 0) + NB(1, -1) - NB(-1, 1) - R(2.0) * NB(-1, 0) - NB(-1, -1));
    R ny = -R(1.0) / (R(8.0) * (R)D.dx[1]) * (NB(1, 1) + R(2.0) * NB(0, 1) + NB(-1, 1) - NB(-1, -1) - R(2.0) * NB(0, -1) - NB(1, -1));
#undef NB
    R norm = sqrt(nx * nx + ny * ny);
    if (norm < R(1E-20)) return 0;
    return d == 0 ? fabs(nx / norm) : fabs(ny / norm);
}

template <typename PT, typename R = typename PT::real>
__device__ inline void thinc_cand(const PT& P, const DevDomain& D, const R* X, long long nt, int i, int j,
                                  int k, int d, ThincCand<R>& t)
{
    const R eps = R(1E-20), beta0 = P.beta;
    int o[3] = {0, 0, 0};
    o[d] = 1;
    t.flag = 0;
    for (int m = 0; m < P.M; ++m) {
        int a = P.S_ALPHA + m;
        R aL = gv(P, D, X, nt, a, i - o[0], j - o[1], k - o[2]);
        R aR = gv(P, D, X, nt, a, i + o[0], j + o[1], k + o[2]);
        R a0 = gv(P, D, X, nt, a, i, j, k);
        R mn = (aR < aL) ? aR : aL;
        R mx = ((aL < aR) ? aR : aL) - mn;
        R theta = (R)((R(0.0) < aR - aL) - (aR - aL < R(0.0)));
        R C = (mx < eps) ? R(0.0) : (a0 - mn + eps) / (mx + eps);
        R delta = R(1E-4);
        int mixed = (C > delta) && (C < (R(0.999999) - delta)) && ((aR - a0) * (a0 - aL) >= R(0.0));
        t.mixed[m] = mixed;
        t.flag = mixed;  // the last material wins (thinc.cpp:110-114)
        t.L[m] = R(0.0);
        t.Rv[m] = R(0.0);
        if (mixed) {
            R nvc = (P.dim == 2) ? youngs(P, D, X, nt, m, i, j, k, d) : R(1.0);
            R beta = nvc * beta0 + R(0.01);
            R coshB = tjm_cosh(beta), tanhB = tjm_tanh(beta);
            R B = tjm_exp(theta * beta * ((R(2.0) * C) - R(1.0)));
            R A = ((B / coshB) - R(1.0)) / tanhB;
            t.Rv[m] = mn + (mx / R(2.0)) * (R(1.0) + theta * ((tanhB + A) / (R(1.0) + A * tanhB)));
            t.L[m] = mn + (mx / R(2.0)) * (R(1.0) + theta * A);
        }
    }
}

// ---------------------------------------------------------------------------
// Reconstruction of one direction.
// ---------------------------------------------------------------------------
// DC >= 0: the direction as a compile-time constant (d is then ignored).
template <typename PT, int DC = -1, typename R = typename PT::real>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1)
    k_recon(PT P, PathBufs<typename PT::real> b, const R* __restrict__ X, int dyn_d)
{
    const int d = DC >= 0 ? DC : dyn_d;
    if (b.scal->done) return;
    const long long nt = b.ntot;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        const int q = find_dom(b.doms, b.ndom, g);
        const DevDomain D = b.doms[q];
        long long l = g - D.off;
        int i, j, k;
        split3(l, D.n[0], D.n[1], i, j, k);
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int rm[3], rp[3];
        long long gm = map_cell(P, D, i - o[0], j - o[1], k - o[2], rm);
        long long gp = map_cell(P, D, i + o[0], j + o[1], k + o[2], rp);
        CellT<R> um, u0, up, L, Rc;
        load_prims(P, X, nt, gm, rm, um);
        load_prims(P, X, nt, g, nullptr, u0);
        load_prims(P, X, nt, gp, rp, up);
        L = u0;
        Rc = u0;
        if (P.muscl) {  // MUSCLextrapolate over the primitive list
            for (int m = 0; m < P.M; ++m) {
                muscl1(um.alpha[m], u0.alpha[m], up.alpha[m], L.alpha[m], Rc.alpha[m]);
                muscl1(um.rhok[m], u0.rhok[m], up.rhok[m], L.rhok[m], Rc.rhok[m]);
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) muscl1(um.vel[r], u0.vel[r], up.vel[r], L.vel[r], Rc.vel[r]);
            muscl1(um.p, u0.p, up.p, L.p, Rc.p);
            if (P.solid)
#pragma unroll
                for (int qq = 0; qq < 9; ++qq) muscl1(um.V[qq], u0.V[qq], up.V[qq], L.V[qq], Rc.V[qq]);
            if (P.plastic)
                for (int m = 0; m < P.M; ++m) muscl1(um.eps[m], u0.eps[m], up.eps[m], L.eps[m], Rc.eps[m]);
            if (P.nmix) muscl1(um.lam, u0.lam, up.lam, L.lam, Rc.lam);
        }
        int reps = 0;
        if (P.thinc) {
            const int* bx = b.boxes + 6 * (D.box_off + b.cell_box[g]);
            int idx[3] = {i, j, k};
            const int in_m = idx[d] - 1 >= bx[d], in_p = idx[d] + 1 <= bx[3 + d];
            reps = D.nbox - b.cell_box[g];
            ThincCand<R> tc, tm, tp;
            thinc_cand(P, D, X, nt, i, j, k, d, tc);
            if (in_m) thinc_cand(P, D, X, nt, i - o[0], j - o[1], k - o[2], d, tm);
            if (in_p) thinc_cand(P, D, X, nt, i + o[0], j + o[1], k + o[2], d, tp);
            const long long gmm = D.off + (i - o[0]) + (long long)D.n[0] * ((j - o[1]) + (long long)D.n[1] * (k - o[2]));
            const long long gpp = D.off + (i + o[0]) + (long long)D.n[0] * ((j + o[1]) + (long long)D.n[1] * (k + o[2]));
            int code = 0;
            for (int m = 0; m < P.M; ++m) {
                const int a = P.S_ALPHA + m;
                R urm, ulp, trm, tlp;
                // UR.left / UL.right: MUSCL value inside the box, stage input in a ghost.
                if (in_m) {
                    R l_, r_;
                    muscl1(gv(P, D, X, nt, a, i - 2 * o[0], j - 2 * o[1], k - 2 * o[2]), um.alpha[m], u0.alpha[m], l_, r_);
                    urm = r_;
                    trm = tm.mixed[m] ? tm.Rv[m] : b.urstar[(long long)m * nt + gmm];
                } else {
                    urm = um.alpha[m];
                    trm = R(0.0);  // URStar ghosts are never written
                }
                if (in_p) {
                    R l_, r_;
                    muscl1(u0.alpha[m], up.alpha[m], gv(P, D, X, nt, a, i + 2 * o[0], j + 2 * o[1], k + 2 * o[2]), l_, r_);
                    ulp = l_;
                    tlp = tp.mixed[m] ? tp.L[m] : b.ulstar[(long long)m * nt + gpp];
                } else {
                    ulp = up.alpha[m];
                    // ULStar's ghost at the box's hi+1 face: star alpha of the last flux pass along d
                    tlp = b.gstar[d][(long long)m * b.nftot[d] + face_index(D, d, i + o[0], j + o[1], k + o[2])];
                }
                R tpl = tc.mixed[m] ? tc.L[m] : b.ulstar[(long long)m * nt + g];
                R tpr = tc.mixed[m] ? tc.Rv[m] : b.urstar[(long long)m * nt + g];
                R upl = L.alpha[m], upr = Rc.alpha[m];
#define MN(x, y) (((y) < (x)) ? (y) : (x))
#define TBV(PL, PR)                                                                                          \
    MN(MN(fabs(urm - (PL)) + fabs((PR)-ulp), fabs(trm - (PL)) + fabs((PR)-tlp)),                            \
       MN(fabs(urm - (PL)) + fabs((PR)-tlp), fabs(trm - (PL)) + fabs((PR)-ulp)))
                R tbvm = TBV(upl, upr);
                R tbvt = TBV(tpl, tpr);
#undef TBV
#undef MN
                if (tc.flag && tbvt < tbvm) {
                    L.alpha[m] = tpl;
                    Rc.alpha[m] = tpr;
                    code |= (tc.mixed[m] ? 1 : 2) << (2 * m);
                }
            }
            if (b.rec) {
                for (int m = 0; m < P.M; ++m) {
                    b.rec[((long long)(d * 2) * P.M + m) * nt + g] = L.alpha[m];
                    b.rec[((long long)(d * 2 + 1) * P.M + m) * nt + g] = Rc.alpha[m];
                }
                b.rec_code[(long long)d * nt + g] = code;
            }
            // THINC pass 1 writes its candidates into the persistent scratch.
            for (int m = 0; m < P.M; ++m)
                if (tc.mixed[m]) {
                    b.ulstar[(long long)m * nt + g] = tc.L[m];
                    b.urstar[(long long)m * nt + g] = tc.Rv[m];
                }
        }
        if (compact_faces(P)) {  // closed by the flux kernel
            store_prim_face(P, b.UL, nt, g, L);
            store_prim_face(P, b.UR, nt, g, Rc);
            continue;
        }
        // cleanUpAlpha of UL and UR: nbox-b times for box b, the closures see
        // the first (hllc.cpp:628-638).
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            CellT<R>& S = side ? Rc : L;
            if (reps > 0) {
                int e = cleanup_alpha(P, S.alpha);
                if (e) set_status(b.scal, e);
            }
            p2c(P, S);
            S.a = sound_speed(P, S);
            for (int r = 1; r < reps; ++r) {
                R before[TJ_MAX_MAT];
                for (int m = 0; m < P.M; ++m) before[m] = S.alpha[m];
                int e = cleanup_alpha(P, S.alpha);
                if (e) set_status(b.scal, e);
                bool same = true;
                for (int m = 0; m < P.M; ++m)
                    same &= same_bits(before[m], S.alpha[m]);
                if (same) break;
            }
        }
        store_face(P, b.UL, nt, g, L);
        store_face(P, b.UR, nt, g, Rc);
    }
}

// ---------------------------------------------------------------------------
// Riemann solvers (hllc.cpp:1-487, flux.cpp:5-47).
// ---------------------------------------------------------------------------
template <typename PT, typename R = typename PT::real>
__device__ inline void star_state(const PT& P, const CellT<R>& U, CellT<R>& Us, R SK, R Ss, int d)  // :12-73
{
    const R tol = R(1E-20);
    R ud = U.vel[d];
    R mult = (fabs((Ss - ud) / Ss) < tol ? R(1.0) : (SK - ud) / (SK - Ss));
    Us.rho = R(0.0);
    for (int m = 0; m < P.M; ++m) {
        Us.alpha[m] = U.alpha[m];
        Us.arho[m] = mult * U.arho[m];
        Us.rhok[m] = Us.arho[m] / Us.alpha[m];
        if (P.nmix && m == 0) Us.arl = mult * U.arl;
        // a fluid carries no plastic strain: its alphaRhoEps star value is 0
        // (the reference writes only the plastic materials' and resets the
        // fluids' after every step, so no result depends on it)
        if (P.plastic) Us.are[m] = P.phase[m] == TJ_PHASE_SOLID ? mult * U.are[m] : R(0.0);
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

// The conservative variables of one state, or their fluxes, by name: kept in
// registers; the flux-word layout is applied only where a face is stored.
template <typename R>
struct FluxV {
    R alpha[TJ_MAX_MAT], arho[TJ_MAX_MAT], rhou[3], E, V[9], are[TJ_MAX_MAT], arl;
};

// Physical flux of the conservative variables (flux.cpp:33-47).
template <typename PT, typename R = typename PT::real>
__device__ inline void phys_flux(const PT& P, const CellT<R>& U, int d, FluxV<R>& F)
{
    R ud = U.vel[d];
    for (int m = 0; m < P.M; ++m) {
        F.alpha[m] = U.alpha[m] * ud;
        F.arho[m] = U.arho[m] * ud;
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) F.rhou[r] = U.rhou[r] * ud - U.sigma[3 * r + d];
    R vs = R(0.0);
#pragma unroll
    for (int i = 0; i < 3; ++i) vs += U.vel[i] * U.sigma[3 * i + d];
    F.E = U.E * ud - vs;
    if (P.solid)
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            int row = q / 3, col = q % 3;
            F.V[q] = U.V[q] * ud - U.V[3 * d + col] * U.vel[row];
        }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) F.are[m] = U.are[m] * ud;
    if (P.nmix) F.arl = U.arl * ud;
}

// Conservative values of a state.
template <typename PT, typename R = typename PT::real>
__device__ inline void cons_vals(const PT& P, const CellT<R>& U, FluxV<R>& Q)
{
    for (int m = 0; m < P.M; ++m) {
        Q.alpha[m] = U.alpha[m];
        Q.arho[m] = U.arho[m];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) Q.rhou[r] = U.rhou[r];
    Q.E = U.E;
    if (P.solid)
#pragma unroll
        for (int q = 0; q < 9; ++q) Q.V[q] = U.V[q];
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) Q.are[m] = U.are[m];
    if (P.nmix) Q.arl = U.arl;
}

// The face flux of every conservative variable but alpha, in the reference's
// evaluation order (hllc.cpp:416-476, 287-371):
//   NT = 0: FK
//   NT = 1: FK + S1 (Q1 - Q0)
//   NT = 2: FK + S1 (Q1 - Q0) + S2 (Q2 - Q1)
// alpha takes the flux of the star state FA.
template <int NT, typename PT, typename R = typename PT::real>
__device__ inline void flux_combine(const PT& P, FluxV<R>& F, const FluxV<R>& FA, const FluxV<R>& FK,
                                    const FluxV<R>& Q0, const FluxV<R>& Q1, const FluxV<R>& Q2, R S1, R S2)
{
    auto one = [&](R fk, R q0, R q1, R q2) -> R {
        if constexpr (NT == 0) return fk;
        else if constexpr (NT == 1) return fk + S1 * (q1 - q0);
        else return fk + S1 * (q1 - q0) + S2 * (q2 - q1);
    };
    for (int m = 0; m < P.M; ++m) {
        F.alpha[m] = FA.alpha[m];
        F.arho[m] = one(FK.arho[m], Q0.arho[m], Q1.arho[m], Q2.arho[m]);
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) F.rhou[r] = one(FK.rhou[r], Q0.rhou[r], Q1.rhou[r], Q2.rhou[r]);
    F.E = one(FK.E, Q0.E, Q1.E, Q2.E);
    if (P.solid)
#pragma unroll
        for (int q = 0; q < 9; ++q) F.V[q] = one(FK.V[q], Q0.V[q], Q1.V[q], Q2.V[q]);
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) F.are[m] = one(FK.are[m], Q0.are[m], Q1.are[m], Q2.are[m]);
    if (P.nmix) F.arl = one(FK.arl, Q0.arl, Q1.arl, Q2.arl);
}

// One face into the flux-word layout (nf faces per word).
template <typename PT, typename R = typename PT::real>
__device__ inline void store_flux(const PT& P, R* FX, long long nf, long long f, const FluxV<R>& F, R Ss,
                                  const R* vstar)
{
#define FXS(w) FX[(long long)(w) * nf + f]
    for (int m = 0; m < P.M; ++m) {
        FXS(P.X_ALPHA + m) = F.alpha[m];
        FXS(P.X_ARHO + m) = F.arho[m];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) FXS(P.X_RHOU + r) = F.rhou[r];
    FXS(P.X_E) = F.E;
    if (P.solid) {
#pragma unroll
        for (int q = 0; q < 9; ++q) FXS(P.X_V + q) = F.V[q];
#pragma unroll
        for (int col = 0; col < 3; ++col) FXS(P.X_VSTAR + col) = vstar[col];
    }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) FXS(P.X_ARE + m) = F.are[m];
    if (P.nmix) FXS(P.X_ARL) = F.arl;
    FXS(P.X_SSTAR) = Ss;
#undef FXS
}

// HLLC (hllc.cpp:384-487) or the 5-wave solver (133-380) at one face. F gets
// the conservative fluxes, Ss the contact speed, vstar the VSTAR(d, col)
// values (solids). Returns the side whose star alpha the face carries: 0
// left, 1 right.
template <typename PT, typename R = typename PT::real>
__device__ inline int face_flux(const PT& P, const CellT<R>& L, const CellT<R>& Rc, int d, FluxV<R>& F, R& Ss,
                                R* vstar, DevScalars* scal)
{
    R x1 = fabs(L.vel[d]) + L.a, x2 = fabs(Rc.vel[d]) + Rc.a;
    R SR = (x1 < x2) ? x2 : x1;
    R SL = -SR;
    Ss = (-Rc.sigma[4 * d] + L.sigma[4 * d] + L.rhou[d] * (SL - L.vel[d]) - Rc.rhou[d] * (SR - Rc.vel[d])) /
         (L.rho * (SL - L.vel[d]) - Rc.rho * (SR - Rc.vel[d]));  // getSstar, hllc.cpp:5-8
    if (!P.solid) {
        // the state K of the upwind side and its star state (no pointer or
        // reference selects between L and Rc: both stay in registers)
        auto hllc_side = [&](const CellT<R>& K, R SK, bool hllc) {
            CellT<R> Ks;
            star_state(P, K, Ks, SK, Ss, d);
            FluxV<R> FK, FS, QK, QS;
            phys_flux(P, K, d, FK);
            phys_flux(P, Ks, d, FS);
            if (hllc) {
                cons_vals(P, K, QK);
                cons_vals(P, Ks, QS);
                flux_combine<1>(P, F, FS, FK, QK, QS, QS, SK, R(0.0));
            } else {
                flux_combine<0>(P, F, FS, FK, FK, FK, FK, R(0.0), R(0.0));
            }
        };
        if (SL >= R(0.0) || Ss >= R(0.0)) {
            hllc_side(L, SL, !(SL >= R(0.0)));
            return 0;
        }
        hllc_side(Rc, SR, SR >= R(0.0));
        return 1;
    }
    CellT<R> Ls, Rs;

    // 5-wave solver for solids (hllc.cpp:133-380).
    if (isnan(SL) || isnan(SR) || isnan(Ss)) { set_status(scal, TJ_ERR_WAVESPEED); return 0; }
    R SLT = R(0.0), SRT = R(0.0);
    CellT<R> Uss;
    FluxV<R> QK, QKs, QSS, FK, FAs;
    int side;
    auto vstar_of = [&](const CellT<R>& U) {  // VSTAR(d, col), read by update
#pragma unroll
        for (int col = 0; col < 3; ++col) vstar[col] = U.V[3 * d + col];
    };
    auto starstar = [&](const CellT<R>& UK, CellT<R>& UKs, R SKT) {  // getStarStarState, hllc.cpp:87-129
        Uss = UKs;
#pragma unroll
        for (int i = 0; i < 3; ++i)  // getSigmaStar, hllc.cpp:75-83
            UKs.sigma[3 * i + d] =
                (Ls.rho * (Ss - SLT) * Rs.rho * (Ss - SRT) * (L.vel[i] - Rc.vel[i]) + Ls.rho * (Ss - SLT) * Rc.sigma[3 * i + d] -
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
    if (SL >= R(0.0)) {
        star_state(P, L, Ls, SL, Ss, d);
        phys_flux(P, Ls, d, FAs);
        phys_flux(P, L, d, FK);
        flux_combine<0>(P, F, FAs, FK, FK, FK, FK, R(0.0), R(0.0));
        vstar_of(L);
        side = 0;
    } else if (Ss >= R(0.0)) {
        star_state(P, L, Ls, SL, Ss, d);
        SLT = Ss - transverse_speed(P, Ls);
        phys_flux(P, Ls, d, FAs);
        phys_flux(P, L, d, FK);
        cons_vals(P, L, QK);
        cons_vals(P, Ls, QKs);
        if (SLT >= R(0.0)) {
            flux_combine<1>(P, F, FAs, FK, QK, QKs, QKs, SL, R(0.0));
            vstar_of(Ls);
        } else {
            star_state(P, Rc, Rs, SR, Ss, d);
            SRT = Ss + transverse_speed(P, Rs);
            starstar(L, Ls, SLT);
            cons_vals(P, Uss, QSS);
            flux_combine<2>(P, F, FAs, FK, QK, QKs, QSS, SL, SLT);
            vstar_of(Uss);
        }
        side = 0;
    } else if (SR >= R(0.0)) {
        star_state(P, Rc, Rs, SR, Ss, d);
        SRT = Ss + transverse_speed(P, Rs);
        phys_flux(P, Rs, d, FAs);
        phys_flux(P, Rc, d, FK);
        cons_vals(P, Rc, QK);
        cons_vals(P, Rs, QKs);
        if (SRT >= R(0.0)) {
            star_state(P, L, Ls, SL, Ss, d);
            SLT = Ss - transverse_speed(P, Ls);
            starstar(Rc, Rs, SRT);
            cons_vals(P, Uss, QSS);
            flux_combine<2>(P, F, FAs, FK, QK, QKs, QSS, SR, SRT);
            vstar_of(Uss);
        } else {
            flux_combine<1>(P, F, FAs, FK, QK, QKs, QKs, SR, R(0.0));
            vstar_of(Rs);
        }
        side = 1;
    } else {
        star_state(P, Rc, Rs, SR, Ss, d);
        phys_flux(P, Rs, d, FAs);
        phys_flux(P, Rc, d, FK);
        flux_combine<0>(P, F, FAs, FK, FK, FK, FK, R(0.0), R(0.0));
        vstar_of(Rc);
        side = 1;
    }
    if (isnan(SL) || isnan(SR) || isnan(Ss) || isnan(SLT) || isnan(SRT)) set_status(scal, TJ_ERR_WAVESPEED);
    return side;
}

template <typename PT, int DC = -1, typename R = typename PT::real>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1) k_flux(PT P, PathBufs<typename PT::real> b, int dyn_d)
{
    const int d = DC >= 0 ? DC : dyn_d;
    if (b.scal->done) return;
    const long long nt = b.ntot, nf = b.nftot[d];
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x) {
        const int q = find_dom_face(b.doms, b.ndom, d, f);
        const DevDomain D = b.doms[q];
        int nfv[3] = {D.n[0], D.n[1], D.n[2]};
        nfv[d] += 1;
        long long l = f - D.foff[d];
        int i, j, k;
        split3(l, nfv[0], nfv[1], i, j, k);
        int o[3] = {0, 0, 0};
        o[d] = 1;
        int rl[3], rr[3];
        long long gl = map_cell(P, D, i - o[0], j - o[1], k - o[2], rl);
        long long gr = map_cell(P, D, i, j, k, rr);
        CellT<R> L, Rc;
        if (compact_faces(P)) {
            load_prim_face(P, b.UR, nt, gl, rl[d] ? d : -1, L);
            load_prim_face(P, b.UL, nt, gr, rr[d] ? d : -1, Rc);
        } else {
            load_face(P, b.UR, nt, gl, rl[d] ? d : -1, L);
            load_face(P, b.UL, nt, gr, rr[d] ? d : -1, Rc);
        }
        FluxV<R> F;
        R Ss, vstar[3] = {R(0.0), R(0.0), R(0.0)};
        int side = face_flux(P, L, Rc, d, F, Ss, vstar, b.scal);
        store_flux(P, b.FX, nf, f, F, Ss, vstar);
        if (P.thinc) {
            const CellT<R>& src = side ? Rc : L;
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
template <typename PT, typename R = typename PT::real>
__device__ inline int plastic_cell(const PT& P, CellT<R>& c)
{
    R tsolid = R(0.0);
    for (int m = 0; m < P.M; ++m)
        if (P.phase[m] == TJ_PHASE_SOLID) tsolid += c.alpha[m];
    if (tsolid <= R(0.5)) {  // cellIsMostlyFluid
        for (int m = 0; m < P.M; ++m) { c.eps[m] = R(0.0); c.are[m] = R(0.0); }
        return 0;
    }
    hencky(P, c);
    R JT = R(0.0), JB = R(0.0), norm = R(0.0), J, Jn;
    for (int m = 0; m < P.M; ++m) {
        ECellT<R> e = ecell_of(c, m);
        if (P.phase[m] == TJ_PHASE_SOLID) {
            J = sqrt(c.hj2);
            R G = eos_G(P, m, e);
            if (G * J * sqrt(R(3.0)) > P.yield[m]) Jn = P.yield[m] / (sqrt(R(3.0)) * G);
            else Jn = J;
            c.eps[m] += sqrt(R(2.0) / R(3.0)) * (J - Jn);
            c.are[m] = c.eps[m] * c.arho[m];
        } else {
            J = R(0.0);
            Jn = R(0.0);
            c.eps[m] = R(0.0);
            c.are[m] = R(0.0);
        }
        JB += (eos_invG(P, m, e)) * J;
        JT += (eos_invG(P, m, e)) * Jn;
        norm += (eos_invG(P, m, e));
    }
    JB *= R(1.0) / norm;
    JT *= R(1.0) / norm;
    if (JB == R(0.0) && JT == R(0.0)) { JB = R(1.0); JT = R(1.0); }
    R t1[9], t2[9], t2i[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            R& dv = c.devH[3 * r + q];
            if (dv != R(0.0) && JB == R(0.0) && JT != R(0.0)) return TJ_ERR_PLASTIC;
            dv *= JT / JB;
            t1[3 * r + q] = (R)(r == q) + R(0.5) * dv;
            t2[3 * r + q] = (R)(r == q) - R(0.5) * dv;
        }
    invert3(t2, t2i);
    mm3(t2i, t1, c.V);
    return 0;
}

// The radial return of a binary32 cell with its return map in binary64
// (plastic.cpp:83-223): the Hencky strain of V is binary32; J = sqrt(HJ2),
// the projection J -> J_new onto the yield surface, the plastic strain and
// alphaRhoEpsilon, the mixture-weighted scale JTotal / JBefore and the
// scaled devH are binary64 from the binary64 EOS parameters, rounded back
// once; the reconstruction of V from devH and the conservativeToPrimitive
// that follows are binary32 (pressure closure in binary64).
template <typename PT, typename R = typename PT::real>
__device__ inline int plastic_cell_proj64(const PT& P, CellT<R>& c)
{
    const DevParams& PD = P.d;
    R tsolid = R(0.0);
    for (int m = 0; m < P.M; ++m)
        if (P.phase[m] == TJ_PHASE_SOLID) tsolid += c.alpha[m];
    if (tsolid <= R(0.5)) {  // cellIsMostlyFluid
        for (int m = 0; m < P.M; ++m) { c.eps[m] = R(0.0); c.are[m] = R(0.0); }
        return 0;
    }
    hencky(P, c);
    const double hj2 = c.hj2;
    double JT = 0.0, JB = 0.0, norm = 0.0;
    for (int m = 0; m < P.M; ++m) {
        ECellT<double> e;
        e.alpha = c.alpha[m];
        e.arho = c.arho[m];
        e.rhok = c.rhok[m];
        e.p = c.p;
        e.hj2 = hj2;
        e.lam = c.lam;
        e.rm0 = c.rm0;
        e.rm1 = c.rm1;
        double J, Jn;
        if (P.phase[m] == TJ_PHASE_SOLID) {
            J = sqrt(hj2);
            const double G = eos_G(PD, m, e);
            Jn = (G * J * sqrt(3.0) > PD.yield[m]) ? PD.yield[m] / (sqrt(3.0) * G) : J;
            const double eps = (double)c.eps[m] + sqrt(2.0 / 3.0) * (J - Jn);
            c.eps[m] = (R)eps;
            c.are[m] = (R)(eps * (double)c.arho[m]);
        } else {
            J = 0.0;
            Jn = 0.0;
            c.eps[m] = R(0.0);
            c.are[m] = R(0.0);
        }
        const double ig = eos_invG(PD, m, e);
        JB += ig * J;
        JT += ig * Jn;
        norm += ig;
    }
    JB *= 1.0 / norm;
    JT *= 1.0 / norm;
    if (JB == 0.0 && JT == 0.0) { JB = 1.0; JT = 1.0; }
    R t1[9], t2[9], t2i[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            R& dv = c.devH[3 * r + q];
            if (dv != R(0.0) && JB == 0.0 && JT != 0.0) return TJ_ERR_PLASTIC;
            dv = (R)((double)dv * (JT / JB));
            t1[3 * r + q] = (R)(r == q) + R(0.5) * dv;
            t2[3 * r + q] = (R)(r == q) - R(0.5) * dv;
        }
    invert3(t2, t2i);
    mm3(t2i, t1, c.V);
    return 0;
}

template <typename PT, typename R = typename PT::real>
__device__ inline void cleanup_v_cell(const PT& P, CellT<R>& c)
{
    R ta = R(0.0), ts = R(0.0);
    for (int m = 0; m < P.M; ++m) {
        ta += c.alpha[m];
        if (P.phase[m] == TJ_PHASE_SOLID) ts += c.alpha[m];
    }
    R B[9], Sq[9];
    mmT3(c.V, c.V, B);
    sqrtm3(B, Sq);
    R norm = tjm_pow(det3(Sq), -R(1.0) / R(3.0));
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) c.V[3 * r + q] = ((Sq[3 * r + q] * norm * ts) + (R)(r == q) * (ta - ts)) / ta;
}

// contains_nan over the conservative and primitive lists of one cell.
template <typename PT, typename R = typename PT::real>
__device__ inline bool cell_has_nan(const PT& P, const CellT<R>& c)
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
    if (P.nmix) n |= isnan(c.lam) || isnan(c.arl);
    return n;
}

// pressureBased_UpdateMassFraction (reactive.cpp:3-26) for the mixture
// (material 0): alphaRhoLambda after one Euler step of the pressure-based burn
// d(alpha rho lambda)/dt = -20 (alpha rho)^0.5 (alpha rho lambda)^0.5 (p/1e6)^1.2,
// clipped at 0; cells with alpha < 0.5 keep their value.
template <typename R>
__device__ __forceinline__ R reactive_euler(R arl, R arho, R p, R alpha, R dt)
{
    const R sigma = R(20.0), nu = R(0.5), n = R(1.2);
    if (alpha < R(0.5)) return arl;
    R r = arl - (dt) * (sigma * tjm_pow(arho, R(1.0) - nu) * tjm_pow(arl, nu) * tjm_pow((p / R(1E6)), n));
    if (r < R(0.0)) r = R(0.0);
    return r;
}

// reactiveUpdate (reactive.cpp:60-103) on one cell: two Euler steps from the
// same alphaRho, pressure and alpha, averaged with the start value, then
// conservativeToPrimitive. Returns the c2p status.
template <typename PT, typename R = typename PT::real>
__device__ inline int reactive_cell(const PT& P, CellT<R>& c, R dt)
{
    const R a0 = c.arl;
    const R a1 = reactive_euler(a0, c.arho[0], c.p, c.alpha[0], dt);
    const R a2 = reactive_euler(a1, c.arho[0], c.p, c.alpha[0], dt);
    c.arl = (a0 * (R(1.0) / R(2.0))) + (a2 * (R(1.0) / R(2.0)));
    return c2p(P, c);
}

// addGeometricSourceTerm (radial.cpp:5-31) on one cell: every conservative
// variable gains dt * (multiplier / r) * geometricFlux (flux.cpp:51-77), with
// r = (i + 0.5) dx[0] and multiplier -2 in 1-D (spherical symmetry), -1 in 2-D
// and 3-D (cylindrical). `sg` is the stress the reference's state holds at that
// point and the velocity is the cell's; neither changes while the conservative
// variables are updated, so the per-cell order is the reference's.
template <typename PT, typename R = typename PT::real>
__device__ inline void radial_source(const PT& P, CellT<R>& c, const R* sg, int i, double dx0, R dt)
{
    const R inv_r = R(P.dim == 1 ? -2.0 : -1.0) / (((R)i + R(0.5)) * (R)dx0);
    const R s = dt * inv_r;
    const R u = c.vel[0];
    for (int m = 0; m < P.M; ++m) {
        c.alpha[m] += s * R(0.0);
        c.arho[m] += s * (c.arho[m] * u);
    }
    c.rhou[0] += s * (((c.rhou[0] * u) - sg[0]) + sg[8]);
    c.rhou[1] += s * ((c.rhou[1] * u) - sg[1]);
    c.rhou[2] += s * (R(-2.0) * sg[2]);
    R vds = R(0.0);  // vdotsigma (flux.cpp:19-29) along x
#pragma unroll
    for (int r = 0; r < 3; ++r) vds += c.vel[r] * sg[3 * r];
    if constexpr (sizeof(R) == 4) dd_add32(c.E, c.Elo, s * ((c.E * u) - vds));
    else c.E += s * ((c.E * u) - vds);
    if (P.nmix) c.arl += s * (c.arl * u);
    if (P.solid) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const R g = (q < 6) ? (R(1.0) / R(3.0)) * c.V[q] * u : -(R(2.0) / R(3.0)) * c.V[q] * u;
            c.V[q] += s * g;
        }
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) c.are[m] += s * (c.are[m] * u);
    }
}

// ---------------------------------------------------------------------------
// Update of one direction; last direction: c2p; second stage: average and
// the post-advance operators of main.cpp:145-187.
// ---------------------------------------------------------------------------
// Flux words of the two faces of a cell in the face arrays (side 0: the
// face below the cell along d, 1: the face above).
template <typename R>
struct FacePairGlobal {
    const R* FX;
    long long nf, f0, f1;
    __device__ __forceinline__ R operator()(int w, int s) const { return FX[(long long)w * nf + (s ? f1 : f0)]; }
};

// Update of cell g along d from the fluxes of its two faces (FXW(w, side));
// the last direction: c2p; second stage: the average and the post-advance
// operators of main.cpp:145-187.
template <typename PT, typename FA, typename R = typename PT::real>
__device__ __forceinline__ void update_cell(const PT& P, const PathBufs<R>& b, const R* __restrict__ X, R* Y,
                                            long long g, const DevDomain& D, int i, int d, int first, int last,
                                            int finish, R dtdx_num, const FA& FXW)
{
    const long long nt = b.ntot;
    CellT<R> U, Yc;
    load_state(P, X, nt, g, nullptr, U);
    if (first) Yc = U;
    else load_state(P, Y, nt, g, nullptr, Yc);
    const R dtdx = dtdx_num / (R)D.dx[d];
    for (int m = 0; m < P.M; ++m) {
        Yc.alpha[m] += dtdx * (FXW(P.X_ALPHA + m, 0) - FXW(P.X_ALPHA + m, 1) - U.alpha[m] * (FXW(P.X_SSTAR, 0) - FXW(P.X_SSTAR, 1)));
        Yc.arho[m] += dtdx * (FXW(P.X_ARHO + m, 0) - FXW(P.X_ARHO + m, 1));
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) Yc.rhou[r] += dtdx * (FXW(P.X_RHOU + r, 0) - FXW(P.X_RHOU + r, 1));
    if constexpr (sizeof(R) == 4) dd_add32(Yc.E, Yc.Elo, dtdx * (FXW(P.X_E, 0) - FXW(P.X_E, 1)));
    else Yc.E += dtdx * (FXW(P.X_E, 0) - FXW(P.X_E, 1));
    if (P.solid)
#pragma unroll
        for (int qq = 0; qq < 9; ++qq) {
            int row = qq / 3, col = qq % 3;
            Yc.V[qq] += dtdx * (FXW(P.X_V + qq, 0) - FXW(P.X_V + qq, 1) -
                                (R(2.0) / R(3.0)) * U.V[qq] * (FXW(P.X_SSTAR, 0) - FXW(P.X_SSTAR, 1)) +
                                U.vel[row] * (FXW(P.X_VSTAR + col, 0) - FXW(P.X_VSTAR + col, 1)));
        }
    if (P.plastic)
        for (int m = 0; m < P.M; ++m) Yc.are[m] += dtdx * (FXW(P.X_ARE + m, 0) - FXW(P.X_ARE + m, 1));
    if (P.nmix) Yc.arl += dtdx * (FXW(P.X_ARL, 0) - FXW(P.X_ARL, 1));
    if (last) {
        const int ce = c2p(P, Yc);
        if (ce) set_status(b.scal, ce);
        if (finish) {
            const R p_stage = Yc.p;  // U2's pressure, before the average
            // U1 = U*0.5 + U2*0.5 over every carried component (hllc.cpp:705)
            CellT<R> A0;
            load_state(P, b.A, nt, g, nullptr, A0);
            for (int m = 0; m < P.M; ++m) {
                Yc.alpha[m] = (A0.alpha[m] * (R(1.0) / R(2.0))) + (Yc.alpha[m] * (R(1.0) / R(2.0)));
                Yc.arho[m] = (A0.arho[m] * (R(1.0) / R(2.0))) + (Yc.arho[m] * (R(1.0) / R(2.0)));
                Yc.rhok[m] = (A0.rhok[m] * (R(1.0) / R(2.0))) + (Yc.rhok[m] * (R(1.0) / R(2.0)));
                if (P.plastic) {
                    Yc.eps[m] = (A0.eps[m] * (R(1.0) / R(2.0))) + (Yc.eps[m] * (R(1.0) / R(2.0)));
                    Yc.are[m] = (A0.are[m] * (R(1.0) / R(2.0))) + (Yc.are[m] * (R(1.0) / R(2.0)));
                }
            }
            Yc.rho = (A0.rho * (R(1.0) / R(2.0))) + (Yc.rho * (R(1.0) / R(2.0)));
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                Yc.rhou[r] = (A0.rhou[r] * (R(1.0) / R(2.0))) + (Yc.rhou[r] * (R(1.0) / R(2.0)));
                Yc.vel[r] = (A0.vel[r] * (R(1.0) / R(2.0))) + (Yc.vel[r] * (R(1.0) / R(2.0)));
            }
            if constexpr (sizeof(R) == 4) avg_pair32(A0.E, A0.Elo, Yc.E, Yc.Elo);
            else Yc.E = (A0.E * (R(1.0) / R(2.0))) + (Yc.E * (R(1.0) / R(2.0)));
            Yc.p = (A0.p * (R(1.0) / R(2.0))) + (Yc.p * (R(1.0) / R(2.0)));
            if (P.solid) {
#pragma unroll
                for (int qq = 0; qq < 9; ++qq) Yc.V[qq] = (A0.V[qq] * (R(1.0) / R(2.0))) + (Yc.V[qq] * (R(1.0) / R(2.0)));
                Yc.hj2 = (A0.hj2 * (R(1.0) / R(2.0))) + (Yc.hj2 * (R(1.0) / R(2.0)));
            }
            if (P.nmix) {
                Yc.rm0 = (A0.rm0 * (R(1.0) / R(2.0))) + (Yc.rm0 * (R(1.0) / R(2.0)));
                Yc.rm1 = (A0.rm1 * (R(1.0) / R(2.0))) + (Yc.rm1 * (R(1.0) / R(2.0)));
                Yc.lam = (A0.lam * (R(1.0) / R(2.0))) + (Yc.lam * (R(1.0) / R(2.0)));
                Yc.arl = (A0.arl * (R(1.0) / R(2.0))) + (Yc.arl * (R(1.0) / R(2.0)));
            }
            if (finish == 2) {  // advance() alone: the average only
                store_state(P, b.A, nt, g, Yc);
                return;
            }
            if (P.reactive && P.nmix) {  // main.cpp:149-152
                const int re = reactive_cell(P, Yc, dtdx_num);
                if (re) set_status(b.scal, re);
            }
            if (P.plastic) {
                int e;
                if constexpr (sizeof(R) == 4) e = plastic_cell_proj64(P, Yc);
                else e = plastic_cell(P, Yc);
                c2p(P, Yc);
                if (e) set_status(b.scal, e);
            }
            if (P.radial) {
                // the stress the reference's U1 holds here: fresh from the
                // c2p of the plastic or the reactive update, else the
                // average of U's and U2's (fluids only: -p I each,
                // boxaccesscellarray.cpp:204-212)
                const bool fresh = P.plastic || (P.reactive && P.nmix);
                R sg[9];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int qq = 0; qq < 3; ++qq) {
                        const R dl = (R)(r == qq);
                        sg[3 * r + qq] = fresh ? Yc.sigma[3 * r + qq]
                                                   : ((-A0.p * dl) * (R(1.0) / R(2.0))) +
                                                         ((-p_stage * dl) * (R(1.0) / R(2.0)));
                    }
                radial_source(P, Yc, sg, i, D.dx[0], dtdx_num);
                const int rc = c2p(P, Yc);  // geometricSourceTerm (radial.cpp:50)
                if (rc) set_status(b.scal, rc);
            }
            if (P.solid) cleanup_v_cell(P, Yc);
            int e = cleanup_alpha(P, Yc.alpha);
            if (e) set_status(b.scal, e);
            if (b.cell_box[g] == D.nbox - 1 && cell_has_nan(P, Yc)) atomicOr(&b.scal->nan_flag, 1);
            store_state(P, b.A, nt, g, Yc);
            return;
        }
    }
    store_state(P, Y, nt, g, Yc);
}

template <typename PT, int DC = -1, typename R = typename PT::real>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1)
    k_update(PT P, PathBufs<typename PT::real> b, const R* __restrict__ X, R* Y, int dyn_d, int first, int last,
             int finish)
{
    const int d = DC >= 0 ? DC : dyn_d;
    if (b.scal->done) return;
    const long long nt = b.ntot, nf = b.nftot[d];
    const R dtdx_num = b.scal->dt;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        const int q = find_dom(b.doms, b.ndom, g);
        const DevDomain D = b.doms[q];
        long long l = g - D.off;
        int i, j, k;
        split3(l, D.n[0], D.n[1], i, j, k);
        int o[3] = {0, 0, 0};
        o[d] = 1;
        const FacePairGlobal<R> fx{b.FX, nf, face_index(D, d, i, j, k), face_index(D, d, i + o[0], j + o[1], k + o[2])};
        update_cell(P, b, X, Y, g, D, i, d, first, last, finish, dtdx_num, fx);
    }
}

// ---------------------------------------------------------------------------
// CFL (timestep.cpp:7-70) and device-side time bookkeeping (main.cpp:121-143).
// ---------------------------------------------------------------------------
template <typename PT, typename R = typename PT::real>
__global__ void k_cfl(PT P, PathBufs<typename PT::real> b, const R* __restrict__ X)
{
    if (b.scal->done) return;
    const long long nt = b.ntot;
    R mn = R(sizeof(R) == 4 ? 3.0e38 : 1.79769313486231570815e+308);
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        const int q = find_dom(b.doms, b.ndom, g);
        const DevDomain D = b.doms[q];
        CellT<R> c;
        load_state(P, X, nt, g, nullptr, c);
        R a = sound_speed(P, c);
        for (int n = 0; n < P.dim; ++n) {
            R v = (R)D.dx[n] / (a + fabs(c.vel[n]));
            if (v < mn) mn = v;
        }
    }
    for (int s = 16; s > 0; s >>= 1) {
        R o = __shfl_down_sync(0xffffffffu, mn, s);
        if (o < mn) mn = o;
    }
    __shared__ R red[32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) red[w] = mn;
    __syncthreads();
    if (w == 0) {
        mn = (lane < (int)(blockDim.x >> 5)) ? red[lane] : R(sizeof(R) == 4 ? 3.0e38 : 1.79769313486231570815e+308);
        for (int s = 16; s > 0; s >>= 1) {
            R o = __shfl_down_sync(0xffffffffu, mn, s);
            if (o < mn) mn = o;
        }
        if (lane == 0) atomicMin(&b.scal->dtmin_bits, (unsigned long long)__double_as_longlong((double)mn));
    }

}

}  // namespace tj
