// Fused 3-D stage kernel of the per-timestep update for fluids (MUSCL, no
// THINC: the reference's 3-D THINC has no interface normal,
// thinc.cpp:124-127), binary32 with a compensated total energy, over any
// number of independent domains (AMReX boxes that are each their own
// domain) in ONE persistent launch per RK stage.
//
// Work list: every domain is cut into tiles of at most TX x TY x TZ cells
// (the split per axis balances the tile extents, so a 27-cell box becomes
// tiles of 9, not 8+8+8+3); the CTAs of a persistent grid (SM count x resident
// CTAs) walk the list. Per tile, in shared memory:
//   stage : primitives of tile + 2-cell halo (ghosts are the domain's
//           boundary images: foextrap / reflect, main.cpp:124-126) and the
//           conserved words of the output cells (U1 = U, hllc.cpp:583);
//   faces : per direction, one thread per face: MUSCL of the two adjacent
//           cells (hllc.cpp:541-575), primitiveToConservative and
//           getSoundSpeed of both states (hllc.cpp:634-638), HLLC flux
//           (hllc.cpp:384-487); a domain-boundary face takes the boundary
//           image of the valid cell's reconstructed state (hllc.cpp:642-643);
//   update: per cell, dt/dx (F_lo - F_hi) with the alpha term (hllc.cpp:493-523);
//   finish: conservativeToPrimitive (hllc.cpp:689); in the second stage the
//           RK2 average (hllc.cpp:705), cleanUpAlpha (main.cpp:170), the next
//           step's CFL minimum over all domains (timestep.cpp:36-70) and the
//           NaN check of each domain's last box (main.cpp:183-187).
// The tile shape (TX, TY, TZ) is a template parameter. The boxes fall into
// size classes (up to 16^3 cells, up to 32^3, larger); a host-side autotuner
// times each candidate shape on each class's tiles once and keeps the fastest
// per class, and each class runs as its own persistent launch per stage (the
// environment variable TJ_TILE3D=AxBxC pins one candidate for all classes).
// Results do not depend on the tile shape (every face and cell is computed
// by the same arithmetic whichever tile owns it).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tj_math.cuh"
#include "tj_mixed.cuh"

namespace tj {

namespace {

constexpr int NT3 = 512;

struct M3P {
    int M;
    int lo_bc[3], hi_bc[3];
    float g[TJ_MAX_MAT], ig[TJ_MAX_MAT], pref[TJ_MAX_MAT], eref[TJ_MAX_MAT];
    float cEh[TJ_MAX_MAT], cEl[TJ_MAX_MAT], eEh[TJ_MAX_MAT], eEl[TJ_MAX_MAT];
};

// one tile of one domain
struct Work3 {
    int dom;
    short i0, j0, k0;
    unsigned char ex, ey, ez, pad;
};

// per-domain data the kernels need
struct Dom3 {
    int n[3];
    float idx[3];     // 1 / dx
    float dx[3];
    long long off;
    int last[6];      // the domain's last box, lo and hi (contains_nan)
};

struct M3B {
    float* X[2];
    const Dom3* doms;
    const Work3* work;
    int nwork;
    DevScalars* scal;
    long long N;
};

// word offsets of the carried binary32 state
template <int M> __host__ __device__ constexpr int S3_A(int m) { return m; }
template <int M> __host__ __device__ constexpr int S3_AR(int m) { return M + m; }
template <int M> __host__ __device__ constexpr int S3_RK(int m) { return 2 * M + m; }
template <int M> __host__ __device__ constexpr int S3_RU(int r) { return 3 * M + r; }
template <int M> __host__ __device__ constexpr int S3_U(int r) { return 3 * M + 3 + r; }
template <int M> __host__ __device__ constexpr int S3_EH() { return 3 * M + 6; }
template <int M> __host__ __device__ constexpr int S3_EL() { return 3 * M + 7; }
template <int M> __host__ __device__ constexpr int S3_P() { return 3 * M + 8; }
template <int M> __host__ __device__ constexpr int S3_N() { return 3 * M + 9; }

__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }

template <int M, int TX, int TY, int TZ>
struct Sm3 {
    static constexpr int SX = TX + 4, SY = TY + 4, SZ = TZ + 4;
    static constexpr int SV = SX * SY * SZ;  // staged cells
    static constexpr int CV = TX * TY * TZ;  // output cells
    // faces of each direction (x faces, y faces, z faces of the tile)
    static constexpr int FV0 = (TX + 1) * TY * TZ, FV1 = TX * (TY + 1) * TZ, FV2 = TX * TY * (TZ + 1);
    static constexpr int NP = 2 * M + 4;  // staged primitives: alpha[M], rho_k[M], u[3], p
    static constexpr int NC = 2 * M + 5;  // conserved: alpha[M], alphaRho[M], rhoU[3], E hi, E lo
    static constexpr int NF = 2 * M + 5;  // face flux: alpha[M], alphaRho[M], rhoU[3], E, S*
    static constexpr int P_OFF = 0;
    static constexpr int C_OFF = P_OFF + NP * SV;
    // the face fluxes of all three directions at once: word q of direction d
    // at F_OFF + FD(d) + q * FVd(d) + face
    static constexpr int F_OFF = C_OFF + NC * CV;
    static constexpr int RED_OFF = F_OFF + NF * (FV0 + FV1 + FV2);
    static __host__ __device__ constexpr int FVd(int d) { return d == 0 ? FV0 : (d == 1 ? FV1 : FV2); }
    static __host__ __device__ constexpr int FD(int d) { return d == 0 ? 0 : (d == 1 ? NF * FV0 : NF * (FV0 + FV1)); }
    static constexpr int TOTAL = RED_OFF + 64;
    // a second staging buffer (primitives and conserved words) after TOTAL:
    // the next tile's copies land there while this tile computes
    static constexpr size_t BYTES = sizeof(float) * (TOTAL + F_OFF);
};

// Asynchronous 4-byte global -> shared copies (cp.async, completed in groups).
__device__ __forceinline__ void cp_async4(float* dst, const float* src)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NG>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(NG) : "memory"); }

__device__ __forceinline__ int map3(int i, int n, int lo, int hi, bool& refl)
{
    refl = false;
    int j = i;
    if (i < 0) {
        if (lo == TJ_BC_REFLECTIVE) { refl = true; j = -1 - i; }
        else j = 0;
    } else if (i > n - 1) {
        if (hi == TJ_BC_REFLECTIVE) { refl = true; j = 2 * n - 1 - i; }
        else j = n - 1;
    }
    return j < 0 ? 0 : (j > n - 1 ? n - 1 : j);
}

// MUSCL slope, the division-free form of the van Leer limiter (hllc.cpp:527-568)
__device__ __forceinline__ void muscl3(float um, float u0, float up, float& l, float& r)
{
    const float a = u0 - um, b = up - u0;
    float g = 0.0f;
    if (a * b > 0.0f) g = (fabsf(a) < fabsf(b)) ? a : b;
    l = u0 - 0.5f * g;
    r = u0 + 0.5f * g;
}

__device__ __forceinline__ float two_sum3(float a, float b, float& e)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

__device__ __forceinline__ void dd_add3(float& hi, float& lo, float b)
{
    float e;
    const float s = two_sum3(hi, b, e);
    lo = __fadd_rn(lo, e);
    const float t = __fadd_rn(s, lo);
    lo = __fsub_rn(lo, __fsub_rn(t, s));
    hi = t;
}

__device__ __forceinline__ float two_prod_acc3(float ch, float cl, float x, float& lo)
{
    const float p = ch * x;
    lo += fmaf(ch, x, -p) + cl * x;
    return p;
}

template <int M>
struct FS3 {
    float a[M], ar[M], rho, ru[3], u[3], E, p, c;
};

// primitiveToConservative + getSoundSpeed of a reconstructed state
template <int M>
__device__ __forceinline__ void p2c3(const M3P& P, const float* rk, FS3<M>& s)
{
    s.rho = 0.0f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        s.ar[m] = s.a[m] * rk[m];
        s.rho += s.ar[m];
    }
    float ke = 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        s.ru[r] = s.u[r] * s.rho;
        ke += 0.5f * s.rho * s.u[r] * s.u[r];
    }
    float G = 0.0f, ec = 0.0f, pc = 0.0f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        G += s.a[m] * P.ig[m];
        ec += P.eref[m] * s.ar[m];
        pc += P.pref[m] * s.a[m] * P.ig[m];
    }
    s.E = s.p * G + ec - pc + ke;
    float sa = 0.0f, xt = 0.0f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const float c2 = s.p * (P.g[m] + 1.0f) / rk[m] - P.pref[m] / rk[m];
        const float v = P.ig[m] * c2 * s.ar[m] / s.rho;
        sa += (0.0f < v) ? v : 0.0f;
        xt += P.ig[m] * s.a[m];
    }
    if (sa <= 0.0f) sa = 1e-6f;
    s.c = sqrtf(sa / xt);
}

// HLLC flux along d (hllc.cpp:384-487): F = alpha[M], alphaRho[M], rhoU[3], E, S*
template <int M>
__device__ __forceinline__ void hllc3(const FS3<M>& L, const FS3<M>& R, int d, float* F)
{
    const float x1 = fabsf(L.u[d]) + L.c, x2 = fabsf(R.u[d]) + R.c;
    const float SR = (x1 < x2) ? x2 : x1;
    const float SL = -SR;
    const float Ss = (R.p - L.p + L.ru[d] * (SL - L.u[d]) - R.ru[d] * (SR - R.u[d])) /
                     (L.rho * (SL - L.u[d]) - R.rho * (SR - R.u[d]));
    F[2 * M + 4] = Ss;
    const bool left = (SL >= 0.0f) || (Ss >= 0.0f);
    const bool hllc = left ? !(SL >= 0.0f) : (SR >= 0.0f);
    const FS3<M>& K = left ? L : R;
    const float SK = left ? SL : SR;
    const float uK = K.u[d];
    const float mult = (fabsf((Ss - uK) / Ss) < 1e-20f) ? 1.0f : (SK - uK) / (SK - Ss);
    float rs = 0.0f, ars[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        ars[m] = mult * K.ar[m];
        rs += ars[m];
    }
    float rus[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) rus[r] = (r == d) ? mult * K.rho * Ss : mult * K.ru[r];
    const float usd = rus[d] / rs;
    const float Es = mult * K.rho * (K.E / K.rho + (Ss - uK) * (Ss + K.p / (K.rho * (SK - uK))));
    const float w = hllc ? SK : 0.0f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        F[m] = K.a[m] * usd;
        F[M + m] = K.ar[m] * uK + w * (ars[m] - K.ar[m]);
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) F[2 * M + r] = K.ru[r] * uK + (r == d ? K.p : 0.0f) + w * (rus[r] - K.ru[r]);
    F[2 * M + 3] = (K.E + K.p) * uK + w * (Es - K.E);
}

template <int M>
__device__ __forceinline__ void cleanup3(float* a)
{
    float tot = 0.0f;
    int nan = 0;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        float v = a[m];
        if (isnan(v)) {
            v = 0.0f;
            if (nan == 0) nan = m;
        } else if (v < 0.0f) v = 1e-6f;
        else if (v > 1.0f) v = 1.0f;
        a[m] = v;
        tot += v;
    }
    if (nan > 0) {
        a[nan] = 1.0f - tot;
        tot += a[nan];
    }
    const float it = 1.0f / tot;
#pragma unroll
    for (int m = 0; m < M; ++m) a[m] *= it;
}

// Reconstructed state of staged cell s along d on side (0: UL, 1: UR).
template <int M, int TX, int TY, int TZ>
__device__ __forceinline__ void recon3(const M3P& P, const float* sm, int s, int stride, int side, int d, bool refl,
                                       FS3<M>& S)
{
    using SM = Sm3<M, TX, TY, TZ>;
    float v[SM::NP];
#pragma unroll
    for (int q = 0; q < SM::NP; ++q) {
        const float* Q = sm + SM::P_OFF + q * SM::SV;
        float l, r;
        muscl3(Q[s - stride], Q[s], Q[s + stride], l, r);
        v[q] = side ? r : l;
    }
    float rk[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        S.a[m] = v[m];
        rk[m] = v[M + m];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) S.u[r] = v[2 * M + r];
    if (refl) S.u[d] = -S.u[d];
    S.p = v[2 * M + 3];
    p2c3<M>(P, rk, S);
}

// Issue the copies of one tile's staged primitives (tile + 2-cell halo,
// ghosts at their boundary images) and of its output cells' conserved words
// into the staging buffer at sp. Values arrive unmodified: stage_fix negates
// the reflected velocities once they have landed.
template <int M, int TX, int TY, int TZ>
__device__ void stage_issue(const M3P& P, const Work3& w, const Dom3& D, const float* __restrict__ Xin, long long N,
                            float* sp)
{
    using SM = Sm3<M, TX, TY, TZ>;
    const int ex = w.ex, ey = w.ey, ez = w.ez, i0 = w.i0, j0 = w.j0, k0 = w.k0;
    const int nx = D.n[0], ny = D.n[1], nz = D.n[2];
    const long long off = D.off;
    const int sx = ex + 4, sy = ey + 4, sz = ez + 4;
    for (int t = threadIdx.x; t < sx * sy * sz; t += NT3) {
        const int x = t % sx, y = (t / sx) % sy, z = t / (sx * sy);
        bool rx, ry, rz;
        const int gi = map3(i0 - 2 + x, nx, P.lo_bc[0], P.hi_bc[0], rx);
        const int gj = map3(j0 - 2 + y, ny, P.lo_bc[1], P.hi_bc[1], ry);
        const int gk = map3(k0 - 2 + z, nz, P.lo_bc[2], P.hi_bc[2], rz);
        const long long g = off + gi + (long long)nx * (gj + (long long)ny * gk);
        const int s = x + SM::SX * (y + SM::SY * z);
#pragma unroll
        for (int m = 0; m < M; ++m) {
            cp_async4(sp + SM::P_OFF + m * SM::SV + s, Xin + S3_A<M>(m) * N + g);
            cp_async4(sp + SM::P_OFF + (M + m) * SM::SV + s, Xin + S3_RK<M>(m) * N + g);
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) cp_async4(sp + SM::P_OFF + (2 * M + r) * SM::SV + s, Xin + S3_U<M>(r) * N + g);
        cp_async4(sp + SM::P_OFF + (2 * M + 3) * SM::SV + s, Xin + S3_P<M>() * N + g);
    }
    for (int t = threadIdx.x; t < ex * ey * ez; t += NT3) {
        const int x = t % ex, y = (t / ex) % ey, z = t / (ex * ey);
        const long long g = off + (i0 + x) + (long long)nx * ((j0 + y) + (long long)ny * (k0 + z));
        const int c = x + TX * (y + TY * z);
#pragma unroll
        for (int m = 0; m < M; ++m) {
            cp_async4(sp + SM::C_OFF + m * SM::CV + c, Xin + S3_A<M>(m) * N + g);
            cp_async4(sp + SM::C_OFF + (M + m) * SM::CV + c, Xin + S3_AR<M>(m) * N + g);
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) cp_async4(sp + SM::C_OFF + (2 * M + r) * SM::CV + c, Xin + S3_RU<M>(r) * N + g);
        cp_async4(sp + SM::C_OFF + (2 * M + 3) * SM::CV + c, Xin + S3_EH<M>() * N + g);
        cp_async4(sp + SM::C_OFF + (2 * M + 4) * SM::CV + c, Xin + S3_EL<M>() * N + g);
    }
}

// The second stage's finish averages with U^n (hllc.cpp:705): ask L2 for the
// rows of a tile's output cells in every U^n word when the tile's staging is
// queued, so that they arrive while the tile before it computes.
template <int M>
__device__ __forceinline__ void prefetch_un(const Work3& w, const Dom3& D, const float* __restrict__ Xun, long long N)
{
    const int ey = w.ey, ez = w.ez, ex = w.ex;
    const int nrow = ey * ez;
    for (int t = threadIdx.x; t < S3_N<M>() * nrow * 2; t += NT3) {
        const int q = t / (2 * nrow), r = (t >> 1) % nrow, e = t & 1;
        const int y = r % ey, z = r / ey;
        const long long g = D.off + (w.i0 + e * (ex - 1)) + (long long)D.n[0] * ((w.j0 + y) + (long long)D.n[1] * (w.k0 + z));
        asm volatile("prefetch.global.L2 [%0];\n" ::"l"(Xun + (long long)q * N + g));
    }
}

// The reflect_odd ghosts (FillDomainBoundary) of a landed staging buffer:
// negate the velocity normal to each reflective face the ghost crosses.
// Returns whether the tile reaches a reflective face (the same answer in
// every thread of the block).
template <int M, int TX, int TY, int TZ>
__device__ bool stage_fix(const M3P& P, const Work3& w, const Dom3& D, float* sp)
{
    using SM = Sm3<M, TX, TY, TZ>;
    const int lo[3] = {w.i0, w.j0, w.k0}, ext[3] = {w.ex, w.ey, w.ez};
    bool near = false;
#pragma unroll
    for (int d = 0; d < 3; ++d)
        near |= (P.lo_bc[d] == TJ_BC_REFLECTIVE && lo[d] < 2) ||
                (P.hi_bc[d] == TJ_BC_REFLECTIVE && lo[d] + ext[d] + 2 > D.n[d]);
    if (!near) return false;
    const int sx = w.ex + 4, sy = w.ey + 4, sz = w.ez + 4;
    for (int t = threadIdx.x; t < sx * sy * sz; t += NT3) {
        const int x = t % sx, y = (t / sx) % sy, z = t / (sx * sy);
        bool r3[3];
        map3(w.i0 - 2 + x, D.n[0], P.lo_bc[0], P.hi_bc[0], r3[0]);
        map3(w.j0 - 2 + y, D.n[1], P.lo_bc[1], P.hi_bc[1], r3[1]);
        map3(w.k0 - 2 + z, D.n[2], P.lo_bc[2], P.hi_bc[2], r3[2]);
        const int s = x + SM::SX * (y + SM::SY * z);
#pragma unroll
        for (int r = 0; r < 3; ++r)
            if (r3[r]) sp[SM::P_OFF + (2 * M + r) * SM::SV + s] = -sp[SM::P_OFF + (2 * M + r) * SM::SV + s];
    }
    return true;
}

template <int M, int TX, int TY, int TZ>
__global__ void __launch_bounds__(NT3) k_stage3d(M3P P, M3B b, int stage, int force)
{
    if (!force && b.scal->done) return;
    using SM = Sm3<M, TX, TY, TZ>;
    extern __shared__ __align__(16) unsigned char smraw3[];
    float* sm = reinterpret_cast<float*>(smraw3);
    const float* __restrict__ Xin = b.X[stage];
    float* __restrict__ Xout = b.X[stage == 0 ? 1 : 0];
    const long long N = b.N;
    const float dtf = (float)b.scal->dt;
    float dtmin = 3.0e38f;
    bool nan_seen = false;
    __shared__ Work3 wsh[2];
    __shared__ Dom3 Dsh[2];

    int wi = blockIdx.x;
    if (wi < b.nwork) {
        if (threadIdx.x == 0) {
            wsh[0] = b.work[wi];
            Dsh[0] = b.doms[wsh[0].dom];
        }
        __syncthreads();
        stage_issue<M, TX, TY, TZ>(P, wsh[0], Dsh[0], Xin, N, sm);
        if (stage == 1) prefetch_un<M>(wsh[0], Dsh[0], Xout, N);
    }
    cp_async_commit();
    for (int it = 0; wi < b.nwork; wi += gridDim.x, ++it) {
        const int cur = it & 1, nxt = cur ^ 1;
        float* const sp = sm + (cur ? SM::TOTAL : 0);  // this tile's staging buffer
        const int wn = wi + gridDim.x;
        __syncthreads();  // the previous tile is done with the other buffer and its slot
        if (threadIdx.x == 0 && wn < b.nwork) {
            wsh[nxt] = b.work[wn];
            Dsh[nxt] = b.doms[wsh[nxt].dom];
        }
        __syncthreads();
        if (wn < b.nwork) {
            stage_issue<M, TX, TY, TZ>(P, wsh[nxt], Dsh[nxt], Xin, N, sm + (nxt ? SM::TOTAL : 0));
            if (stage == 1) prefetch_un<M>(wsh[nxt], Dsh[nxt], Xout, N);
        }
        cp_async_commit();
        cp_async_wait<1>();  // this tile's copies have landed
        __syncthreads();
        if (stage_fix<M, TX, TY, TZ>(P, wsh[cur], Dsh[cur], sp)) __syncthreads();
        const Work3& w = wsh[cur];
        const Dom3& D = Dsh[cur];
        const int ex = w.ex, ey = w.ey, ez = w.ez;
        const int i0 = w.i0, j0 = w.j0, k0 = w.k0;
        const long long off = D.off;
        const int nx = D.n[0], ny = D.n[1], nz = D.n[2];

        // ---- faces of all three directions: the update is unsplit, so every
        //      face reads the same staged stage-input state; the faces are dealt
        //      to the threads round-robin over the three directions' list, so
        //      that no thread waits for a second round that only a few need ----
        {
            int base = 0;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int fx = ex + (d == 0), fy = ey + (d == 1), fz = ez + (d == 2);
                const int nfd = fx * fy * fz;
                const int stride = d == 0 ? 1 : (d == 1 ? SM::SX : SM::SX * SM::SY);
                const int n_d = d == 0 ? nx : (d == 1 ? ny : nz);
                const int p0 = d == 0 ? i0 : (d == 1 ? j0 : k0);
                const bool lo_refl = P.lo_bc[d] == TJ_BC_REFLECTIVE, hi_refl = P.hi_bc[d] == TJ_BC_REFLECTIVE;
                int u0 = ((int)threadIdx.x - base) % NT3;
                if (u0 < 0) u0 += NT3;
                for (int t = u0; t < nfd; t += NT3) {
                    const int x = t % fx, y = (t / fx) % fy, z = t / (fx * fy);
                    const int f_d = d == 0 ? x : (d == 1 ? y : z);
                    const int posR = p0 + f_d;  // the face's right cell along d
                    // staged index of the right cell and the left cell
                    const int sR = (x + 2) + SM::SX * ((y + 2) + SM::SY * (z + 2));
                    const int sL = sR - stride;
                    FS3<M> L, R;
                    if (posR == 0) recon3<M, TX, TY, TZ>(P, sp, sR, stride, 1, d, lo_refl, L);  // image of UR(0)
                    else recon3<M, TX, TY, TZ>(P, sp, sL, stride, 1, d, false, L);
                    if (posR == n_d) recon3<M, TX, TY, TZ>(P, sp, sL, stride, 0, d, hi_refl, R);  // image of UL(n-1)
                    else recon3<M, TX, TY, TZ>(P, sp, sR, stride, 0, d, false, R);
                    float F[2 * M + 5];
                    hllc3<M>(L, R, d, F);
                    const int fidx = x + fx * (y + fy * z);
#pragma unroll
                    for (int q = 0; q < 2 * M + 5; ++q) sm[SM::F_OFF + SM::FD(d) + q * SM::FVd(d) + fidx] = F[q];
                }
                base += nfd;
            }
        }
        __syncthreads();

        // ---- per cell: the update of the three directions in order x, y, z
        //      (hllc.cpp:493-523), then the finish; a cell's words are touched
        //      by its own thread only, so no barrier separates the two ----
        for (int t = threadIdx.x; t < ex * ey * ez; t += NT3) {
            const int x = t % ex, y = (t / ex) % ey, z = t / (ex * ey);
            const int c = x + TX * (y + TY * z);
            const int s = (x + 2) + SM::SX * ((y + 2) + SM::SY * (z + 2));
            float* C = sp + SM::C_OFF;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int fx = ex + (d == 0), fy = ey + (d == 1);
                const int f0 = x + fx * (y + fy * z);
                const int f1 = f0 + (d == 0 ? 1 : (d == 1 ? fx : fx * fy));
                const float dtdx = dtf * D.idx[d];
                const float* Fl = sm + SM::F_OFF + SM::FD(d);
                const int fv = SM::FVd(d);
                const float dS = Fl[(2 * M + 4) * fv + f0] - Fl[(2 * M + 4) * fv + f1];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const float a0 = sp[SM::P_OFF + m * SM::SV + s];
                    C[m * SM::CV + c] += dtdx * (Fl[m * fv + f0] - Fl[m * fv + f1] - a0 * dS);
                    C[(M + m) * SM::CV + c] += dtdx * (Fl[(M + m) * fv + f0] - Fl[(M + m) * fv + f1]);
                }
#pragma unroll
                for (int r = 0; r < 3; ++r)
                    C[(2 * M + r) * SM::CV + c] += dtdx * (Fl[(2 * M + r) * fv + f0] - Fl[(2 * M + r) * fv + f1]);
                float eh = C[(2 * M + 3) * SM::CV + c], el = C[(2 * M + 4) * SM::CV + c];
                dd_add3(eh, el, dtdx * (Fl[(2 * M + 3) * fv + f0] - Fl[(2 * M + 3) * fv + f1]));
                C[(2 * M + 3) * SM::CV + c] = eh;
                C[(2 * M + 4) * SM::CV + c] = el;
            }

            // ---- finish ----
            const int gi = i0 + x, gj = j0 + y, gk = k0 + z;
            const long long g = off + gi + (long long)nx * (gj + (long long)ny * gk);
            float a[M], ar[M], rk[M], ru[3], u[3], eh, el, p;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                a[m] = C[m * SM::CV + c];
                ar[m] = C[(M + m) * SM::CV + c];
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) ru[r] = C[(2 * M + r) * SM::CV + c];
            eh = C[(2 * M + 3) * SM::CV + c];
            el = C[(2 * M + 4) * SM::CV + c];
            float rho = 0.0f;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                rk[m] = ar[m] / a[m];
                rho += ar[m];
            }
            float ke = 0.0f;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                u[r] = ru[r] / rho;
                ke += 0.5f * rho * u[r] * u[r];
            }
            // p = (E - KE - sum e_cold + sum p_cold) / sum alpha/Gamma, the
            // numerator as an unevaluated pair (boxaccesscellarray.cpp:116)
            float sh = eh, sl = el, e, lo;
            sh = two_sum3(sh, -ke, e);
            sl += e;
            float G = 0.0f;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                lo = 0.0f;
                const float ec = two_prod_acc3(P.eEh[m], P.eEl[m], ar[m], lo);
                sh = two_sum3(sh, -ec, e);
                sl += e - lo;
                lo = 0.0f;
                const float pc = two_prod_acc3(P.cEh[m], P.cEl[m], a[m], lo);
                sh = two_sum3(sh, pc, e);
                sl += e + lo;
                G += a[m] * P.ig[m];
            }
            p = (sh + sl) / G;
            if (stage == 1) {
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    a[m] = 0.5f * Xout[S3_A<M>(m) * N + g] + 0.5f * a[m];
                    ar[m] = 0.5f * Xout[S3_AR<M>(m) * N + g] + 0.5f * ar[m];
                    rk[m] = 0.5f * Xout[S3_RK<M>(m) * N + g] + 0.5f * rk[m];
                }
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    ru[r] = 0.5f * Xout[S3_RU<M>(r) * N + g] + 0.5f * ru[r];
                    u[r] = 0.5f * Xout[S3_U<M>(r) * N + g] + 0.5f * u[r];
                }
                p = 0.5f * Xout[S3_P<M>() * N + g] + 0.5f * p;
                float hs = 0.5f * Xout[S3_EH<M>() * N + g], ls = 0.5f * Xout[S3_EL<M>() * N + g];
                dd_add3(hs, ls, 0.5f * eh);
                ls = __fadd_rn(ls, 0.5f * el);
                const float tt = __fadd_rn(hs, ls);
                el = __fsub_rn(ls, __fsub_rn(tt, hs));
                eh = tt;
                cleanup3<M>(a);
                float rr = 0.0f, sa = 0.0f, xt = 0.0f;
#pragma unroll
                for (int m = 0; m < M; ++m) rr += ar[m];
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const float c2 = p * (P.g[m] + 1.0f) / rk[m] - P.pref[m] / rk[m];
                    const float v = P.ig[m] * c2 * ar[m] / rr;
                    sa += (0.0f < v) ? v : 0.0f;
                    xt += P.ig[m] * a[m];
                }
                if (sa <= 0.0f) sa = 1e-6f;
                const float cs = sqrtf(sa / xt);
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const float v = D.dx[r] / (cs + fabsf(u[r]));
                    if (v < dtmin) dtmin = v;
                }
                if (gi >= D.last[0] && gi <= D.last[3] && gj >= D.last[1] && gj <= D.last[4] && gk >= D.last[2] &&
                    gk <= D.last[5]) {
                    bool nn = isnan(eh) || isnan(p);
#pragma unroll
                    for (int m = 0; m < M; ++m) nn |= isnan(a[m]) || isnan(ar[m]) || isnan(rk[m]);
#pragma unroll
                    for (int r = 0; r < 3; ++r) nn |= isnan(ru[r]) || isnan(u[r]);
                    nan_seen |= nn;
                }
            }
#pragma unroll
            for (int m = 0; m < M; ++m) {
                Xout[S3_A<M>(m) * N + g] = a[m];
                Xout[S3_AR<M>(m) * N + g] = ar[m];
                Xout[S3_RK<M>(m) * N + g] = rk[m];
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                Xout[S3_RU<M>(r) * N + g] = ru[r];
                Xout[S3_U<M>(r) * N + g] = u[r];
            }
            Xout[S3_EH<M>() * N + g] = eh;
            Xout[S3_EL<M>() * N + g] = el;
            Xout[S3_P<M>() * N + g] = p;
        }
    }
    if (stage == 1 && !force) {
        if (nan_seen) atomicOr(&b.scal->nan_flag, 1);
        for (int o = 16; o > 0; o >>= 1) dtmin = fminf(dtmin, __shfl_down_sync(0xffffffffu, dtmin, o));
        float* red = sm + SM::RED_OFF;
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dtmin;
        __syncthreads();
        if (threadIdx.x == 0) {
            float mn = red[0];
            for (int k = 1; k < NT3 / 32; ++k) mn = fminf(mn, red[k]);
            atomicMin(&b.scal->dtmin_bits, (unsigned long long)__double_as_longlong((double)mn));
        }
    }
}

// CFL of the current state, per tile of the work list.
template <int M>
__global__ void k_cfl3d(M3P P, M3B b)
{
    float dtmin = 3.0e38f;
    const long long N = b.N;
    const float* X = b.X[0];
    for (int wi = blockIdx.x; wi < b.nwork; wi += gridDim.x) {
        const Work3 w = b.work[wi];
        const Dom3 D = b.doms[w.dom];
        for (int t = threadIdx.x; t < w.ex * w.ey * w.ez; t += blockDim.x) {
            const int x = t % w.ex, y = (t / w.ex) % w.ey, z = t / (w.ex * w.ey);
            const long long g = D.off + (w.i0 + x) + (long long)D.n[0] * ((w.j0 + y) + (long long)D.n[1] * (w.k0 + z));
            float rr = 0.0f, sa = 0.0f, xt = 0.0f, a[M], ar[M], rk[M];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                a[m] = X[S3_A<M>(m) * N + g];
                ar[m] = X[S3_AR<M>(m) * N + g];
                rk[m] = X[S3_RK<M>(m) * N + g];
                rr += ar[m];
            }
            const float p = X[S3_P<M>() * N + g];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const float c2 = p * (P.g[m] + 1.0f) / rk[m] - P.pref[m] / rk[m];
                const float v = P.ig[m] * c2 * ar[m] / rr;
                sa += (0.0f < v) ? v : 0.0f;
                xt += P.ig[m] * a[m];
            }
            if (sa <= 0.0f) sa = 1e-6f;
            const float cs = sqrtf(sa / xt);
#pragma unroll
            for (int r = 0; r < 3; ++r) dtmin = fminf(dtmin, D.dx[r] / (cs + fabsf(X[S3_U<M>(r) * N + g])));
        }
    }
    for (int o = 16; o > 0; o >>= 1) dtmin = fminf(dtmin, __shfl_down_sync(0xffffffffu, dtmin, o));
    if ((threadIdx.x & 31) == 0) atomicMin(&b.scal->dtmin_bits, (unsigned long long)__double_as_longlong((double)dtmin));
}

template <int M>
__global__ void k_from_fp64_3d(DevParams DP, M3B b, const double* A)
{
    const long long N = b.N;
    float* X = b.X[0];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int m = 0; m < M; ++m) {
            X[S3_A<M>(m) * N + g] = (float)A[(DP.S_ALPHA + m) * N + g];
            X[S3_AR<M>(m) * N + g] = (float)A[(DP.S_ARHO + m) * N + g];
            X[S3_RK<M>(m) * N + g] = (float)A[(DP.S_RHOK + m) * N + g];
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            X[S3_RU<M>(r) * N + g] = (float)A[(DP.S_RHOU + r) * N + g];
            X[S3_U<M>(r) * N + g] = (float)A[(DP.S_VEL + r) * N + g];
        }
        const double E = A[DP.S_E * N + g];
        const float eh = (float)E;
        X[S3_EH<M>() * N + g] = eh;
        X[S3_EL<M>() * N + g] = (float)(E - (double)eh);
        X[S3_P<M>() * N + g] = (float)A[DP.S_P * N + g];
    }
}

template <int M>
__global__ void k_to_fp64_3d(DevParams DP, M3B b, double* A)
{
    const long long N = b.N;
    const float* X = b.X[0];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        double rho = 0.0;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            A[(DP.S_ALPHA + m) * N + g] = X[S3_A<M>(m) * N + g];
            A[(DP.S_ARHO + m) * N + g] = X[S3_AR<M>(m) * N + g];
            A[(DP.S_RHOK + m) * N + g] = X[S3_RK<M>(m) * N + g];
            rho += (double)X[S3_AR<M>(m) * N + g];
        }
        A[DP.S_RHO * N + g] = rho;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            A[(DP.S_RHOU + r) * N + g] = X[S3_RU<M>(r) * N + g];
            A[(DP.S_VEL + r) * N + g] = X[S3_U<M>(r) * N + g];
        }
        A[DP.S_E * N + g] = (double)X[S3_EH<M>() * N + g] + (double)X[S3_EL<M>() * N + g];
        A[DP.S_P * N + g] = X[S3_P<M>() * N + g];
    }
}

__global__ void k_reset_dtmin3(DevScalars* s)
{
    if (threadIdx.x == 0) s->dtmin_bits = 0x7FEFFFFFFFFFFFFFull;
}

inline int nblk3(long long n) { return (int)std::min<long long>((n + 255) / 256, 152 * 8); }

// Cut extent L into pieces of at most T, as even as possible.
void split_axis(int L, int T, std::vector<std::pair<int, int>>& out)
{
    const int k = (L + T - 1) / T;
    out.clear();
    int s = 0;
    for (int q = 0; q < k; ++q) {
        const int e = L / k + (q < L % k ? 1 : 0);
        out.push_back({s, e});
        s += e;
    }
}

// One tile shape: launch helpers of one template instance.
struct Shape {
    int tx, ty, tz;
    size_t smem;
    void (*stage)(const M3P&, const M3B&, int, int, int, size_t, cudaStream_t);
    int (*occupancy)(size_t);
};

template <int M, int TX, int TY, int TZ>
void stage_launch(const M3P& P, const M3B& b, int stage, int force, int grid, size_t smem, cudaStream_t st)
{
    k_stage3d<M, TX, TY, TZ><<<grid, NT3, smem, st>>>(P, b, stage, force);
}

template <int M, int TX, int TY, int TZ>
int stage_occupancy(size_t smem)
{
    // a shape whose shared memory exceeds the opt-in maximum cannot run here:
    // 0, with the error the attribute call raised cleared
    if (cudaFuncSetAttribute(k_stage3d<M, TX, TY, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_stage3d<M, TX, TY, TZ>, NT3, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nb;
}

template <int M, int TX, int TY, int TZ>
Shape make_shape()
{
    return Shape{TX, TY, TZ, Sm3<M, TX, TY, TZ>::BYTES, stage_launch<M, TX, TY, TZ>, stage_occupancy<M, TX, TY, TZ>};
}

template <int M>
std::vector<Shape> shapes()
{
    return {make_shape<M, 8, 8, 8>(), make_shape<M, 8, 8, 4>(), make_shape<M, 16, 8, 4>(), make_shape<M, 16, 4, 4>(),
            make_shape<M, 4, 4, 4>()};
}

// Box-size classes of the autotuner, by valid-cell count: small boxes up to
// 16^3 cells, medium up to 32^3, large above. Each class gets its own tile
// shape, chosen by timing, and its own persistent launch per RK stage: the
// boxes are independent domains, so the classes' launches need no ordering
// among themselves beyond the stream's.
constexpr int kClasses = 3;
constexpr long long kClassMaxCells[kClasses - 1] = {16LL * 16 * 16, 32LL * 32 * 32};
constexpr const char* kClassName[kClasses] = {"small", "medium", "large"};

inline int box_class(const DevDomain& D)
{
    const long long v = (long long)D.n[0] * D.n[1] * D.n[2];
    int c = 0;
    while (c < kClasses - 1 && v > kClassMaxCells[c]) ++c;
    return c;
}

// The tiles of one class under one tile shape, on the device.
struct ClassPlan {
    std::vector<int> doms;  // domains of the class
    int best = -1;          // chosen shape
    int grid = 0;
    Work3* d_work = nullptr;
    int nwork = 0;
    long long cells = 0;
    std::vector<double> tune_ms;
};

struct Mixed3D : MixedBase {
    M3P P;
    M3B b;
    int M = 0;
    float* X[2] = {nullptr, nullptr};
    Dom3* d_doms = nullptr;
    Work3* d_work = nullptr;  // every tile of every class (the CFL pass)
    std::vector<Shape> cand;
    std::vector<int> occ;  // resident CTAs per SM of each candidate (0: does not fit)
    ClassPlan cls[kClasses];
    bool tuned = false;
    int sms = 0;
    long long N = 0;
    std::vector<DevDomain> hdoms;
    std::vector<std::vector<int>> hboxes;

    ~Mixed3D() override
    {
        if (X[0]) cudaFree(X[0]);
        if (X[1]) cudaFree(X[1]);
        if (d_doms) cudaFree(d_doms);
        if (d_work) cudaFree(d_work);
        for (auto& c : cls)
            if (c.d_work) cudaFree(c.d_work);
    }

    int alloc(const DevParams& DP, const std::vector<DevDomain>& doms, long long ntot, cudaStream_t st)
    {
        M = DP.M;
        N = ntot;
        std::memset(&P, 0, sizeof P);
        P.M = M;
        for (int d = 0; d < 3; ++d) {
            P.lo_bc[d] = DP.lo_bc[d];
            P.hi_bc[d] = DP.hi_bc[d];
        }
        for (int k = 0; k < M; ++k) {
            const double G = DP.prm[k][0] - 1.0;
            P.g[k] = (float)G;
            P.ig[k] = (float)(1.0 / G);
            P.pref[k] = (float)DP.prm[k][1];
            P.eref[k] = (float)DP.prm[k][2];
            const double cE = DP.prm[k][1] / G, eE = DP.prm[k][2];
            P.cEh[k] = (float)cE;
            P.cEl[k] = (float)(cE - (double)P.cEh[k]);
            P.eEh[k] = (float)eE;
            P.eEl[k] = (float)(eE - (double)P.eEh[k]);
        }
        const int NW = S3_N<4>() - 3 * (4 - M);  // 3M + 9
        for (int q = 0; q < 2; ++q) {
            if (cudaMalloc(&X[q], sizeof(float) * NW * N) != cudaSuccess) return TJ_ERR_CUDA;
            cudaMemsetAsync(X[q], 0, sizeof(float) * NW * N, st);
        }
        switch (M) {
            case 1: cand = shapes<1>(); break;
            case 2: cand = shapes<2>(); break;
            case 3: cand = shapes<3>(); break;
            default: cand = shapes<4>(); break;
        }
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        occ.clear();
        for (const Shape& S : cand) occ.push_back(S.occupancy(S.smem));
        b.X[0] = X[0];
        b.X[1] = X[1];
        b.N = N;
        b.scal = nullptr;
        std::vector<std::vector<int>> one(doms.size());
        for (size_t q = 0; q < doms.size(); ++q)
            one[q] = {0, 0, 0, doms[q].n[0] - 1, doms[q].n[1] - 1, doms[q].n[2] - 1};
        return set_boxes(doms, one, st);
    }

    // The tiles of the given domains under shape s, largest first.
    std::vector<Work3> tiles(const std::vector<int>& doms, int s) const
    {
        const Shape& S = cand[s];
        std::vector<Work3> work;
        std::vector<std::pair<int, int>> ax[3];
        for (int q : doms) {
            const DevDomain& D = hdoms[q];
            split_axis(D.n[0], S.tx, ax[0]);
            split_axis(D.n[1], S.ty, ax[1]);
            split_axis(D.n[2], S.tz, ax[2]);
            for (auto& z : ax[2])
                for (auto& y : ax[1])
                    for (auto& x : ax[0]) {
                        Work3 w;
                        w.dom = q;
                        w.i0 = (short)x.first;
                        w.j0 = (short)y.first;
                        w.k0 = (short)z.first;
                        w.ex = (unsigned char)x.second;
                        w.ey = (unsigned char)y.second;
                        w.ez = (unsigned char)z.second;
                        w.pad = 0;
                        work.push_back(w);
                    }
        }
        // largest tiles first: the persistent CTAs balance the tail
        std::stable_sort(work.begin(), work.end(),
                         [](const Work3& a, const Work3& c) { return a.ex * a.ey * a.ez > c.ex * c.ey * c.ez; });
        return work;
    }

    static int upload(Work3*& dst, const std::vector<Work3>& w, cudaStream_t st)
    {
        if (dst) cudaFree(dst);
        dst = nullptr;
        if (cudaMalloc(&dst, sizeof(Work3) * std::max<size_t>(w.size(), 1)) != cudaSuccess) return TJ_ERR_CUDA;
        if (!w.empty()) cudaMemcpyAsync(dst, w.data(), sizeof(Work3) * w.size(), cudaMemcpyHostToDevice, st);
        cudaStreamSynchronize(st);
        return TJ_OK;
    }

    // Whether shape s fits this GPU at this material count (its shared
    // memory at most the opt-in maximum): at least one resident CTA.
    bool fits(int s) const { return occ[s] >= 1; }

    int first_fit() const
    {
        for (size_t s = 0; s < cand.size(); ++s)
            if (fits((int)s)) return (int)s;
        return -1;
    }

    // Class c's work list under shape s, on the device, and its grid.
    int plan_class(int c, int s, cudaStream_t st)
    {
        if (s < 0 || !fits(s)) return TJ_ERR_ARG;
        ClassPlan& C = cls[c];
        const std::vector<Work3> w = tiles(C.doms, s);
        if (int e = upload(C.d_work, w, st)) return e;
        C.nwork = (int)w.size();
        C.best = s;
        C.grid = std::max(1, std::min(C.nwork, sms * occ[s]));
        return TJ_OK;
    }

    // The CFL pass's work list: every tile of every class under its shape.
    int plan_all(cudaStream_t st)
    {
        std::vector<Work3> all;
        for (int c = 0; c < kClasses; ++c) {
            if (cls[c].doms.empty()) continue;
            const std::vector<Work3> w = tiles(cls[c].doms, cls[c].best >= 0 ? cls[c].best : std::max(0, first_fit()));
            all.insert(all.end(), w.begin(), w.end());
        }
        if (int e = upload(d_work, all, st)) return e;
        b.work = d_work;
        b.nwork = (int)all.size();
        return TJ_OK;
    }

    M3B class_bufs(int c) const
    {
        M3B bc = b;
        bc.work = cls[c].d_work;
        bc.nwork = cls[c].nwork;
        return bc;
    }

    int set_boxes(const std::vector<DevDomain>& doms, const std::vector<std::vector<int>>& boxes,
                  cudaStream_t st) override
    {
        hdoms = doms;
        hboxes = boxes;
        std::vector<Dom3> d3(doms.size());
        for (auto& c : cls) {
            c.doms.clear();
            c.cells = 0;
        }
        for (size_t q = 0; q < doms.size(); ++q) {
            const DevDomain& D = doms[q];
            for (int k = 0; k < 3; ++k) {
                if (D.n[k] > 32000) return TJ_ERR_ARG;  // tile origins are 16-bit
                d3[q].n[k] = D.n[k];
                d3[q].dx[k] = (float)D.dx[k];
                d3[q].idx[k] = (float)(1.0 / D.dx[k]);
            }
            d3[q].off = D.off;
            const std::vector<int>& bl = boxes[q];
            const int* L = &bl[bl.size() - 6];
            for (int k = 0; k < 6; ++k) d3[q].last[k] = L[k];
            ClassPlan& C = cls[box_class(D)];
            C.doms.push_back((int)q);
            C.cells += (long long)D.n[0] * D.n[1] * D.n[2];
        }
        if (d_doms) cudaFree(d_doms);
        d_doms = nullptr;
        if (cudaMalloc(&d_doms, sizeof(Dom3) * d3.size()) != cudaSuccess) return TJ_ERR_CUDA;
        cudaMemcpyAsync(d_doms, d3.data(), sizeof(Dom3) * d3.size(), cudaMemcpyHostToDevice, st);
        b.doms = d_doms;
        tuned = false;  // re-tune on the next upload
        const int s0 = first_fit();
        if (s0 < 0) return TJ_ERR_ARG;
        for (int c = 0; c < kClasses; ++c)
            if (!cls[c].doms.empty())
                if (int e = plan_class(c, s0, st)) return e;
        return plan_all(st);
    }

    // For each box-size class, times one stage launch per candidate shape
    // over that class's tiles on the current state and keeps the fastest
    // (the trial results are discarded: the stage-1 output buffer is scratch
    // until the next step). TJ_TILE3D=AxBxC pins one candidate for every
    // class instead.
    void autotune(cudaStream_t st)
    {
        int pinned = -1;
        if (const char* env = std::getenv("TJ_TILE3D")) {
            int a = 0, c = 0, d = 0;
            if (std::sscanf(env, "%dx%dx%d", &a, &c, &d) == 3)
                for (size_t s = 0; s < cand.size(); ++s)
                    if (cand[s].tx == a && cand[s].ty == c && cand[s].tz == d) pinned = (int)s;
        }
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (int c = 0; c < kClasses; ++c) {
            ClassPlan& C = cls[c];
            if (C.doms.empty()) continue;
            if (pinned >= 0 && plan_class(c, pinned, st) == TJ_OK) continue;
            C.tune_ms.assign(cand.size(), 0.0);
            float bestms = 3e38f;
            int bi = first_fit();
            for (size_t s = 0; s < cand.size(); ++s) {
                if (plan_class(c, (int)s, st) != TJ_OK) continue;
                const M3B bc = class_bufs(c);
                cand[s].stage(P, bc, 0, 1, C.grid, cand[s].smem, st);  // warm-up
                cudaEventRecord(e0, st);
                for (int r = 0; r < 3; ++r) cand[s].stage(P, bc, 0, 1, C.grid, cand[s].smem, st);
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                C.tune_ms[s] = ms / 3.0;
                if (ms < bestms) {
                    bestms = ms;
                    bi = (int)s;
                }
            }
            plan_class(c, bi, st);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        plan_all(st);
        tuned = true;
        cudaGetLastError();
    }

    int from_fp64(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st) override
    {
        b.scal = fb.scal;
        switch (M) {
            case 1: k_from_fp64_3d<1><<<nblk3(N), 256, 0, st>>>(DP, b, fb.A); break;
            case 2: k_from_fp64_3d<2><<<nblk3(N), 256, 0, st>>>(DP, b, fb.A); break;
            case 3: k_from_fp64_3d<3><<<nblk3(N), 256, 0, st>>>(DP, b, fb.A); break;
            default: k_from_fp64_3d<4><<<nblk3(N), 256, 0, st>>>(DP, b, fb.A); break;
        }
        if (!tuned) autotune(st);
        return 1 + cfl(fb, st);
    }

    int to_fp64(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st) override
    {
        switch (M) {
            case 1: k_to_fp64_3d<1><<<nblk3(N), 256, 0, st>>>(DP, b, fb.A); break;
            case 2: k_to_fp64_3d<2><<<nblk3(N), 256, 0, st>>>(DP, b, fb.A); break;
            case 3: k_to_fp64_3d<3><<<nblk3(N), 256, 0, st>>>(DP, b, fb.A); break;
            default: k_to_fp64_3d<4><<<nblk3(N), 256, 0, st>>>(DP, b, fb.A); break;
        }
        return 1;
    }

    int cfl(const Fp64Bufs& fb, cudaStream_t st) override
    {
        b.scal = fb.scal;
        k_reset_dtmin3<<<1, 32, 0, st>>>(fb.scal);
        const int g = std::max(1, std::min(b.nwork, 152 * 8));
        switch (M) {
            case 1: k_cfl3d<1><<<g, 256, 0, st>>>(P, b); break;
            case 2: k_cfl3d<2><<<g, 256, 0, st>>>(P, b); break;
            case 3: k_cfl3d<3><<<g, 256, 0, st>>>(P, b); break;
            default: k_cfl3d<4><<<g, 256, 0, st>>>(P, b); break;
        }
        return 2;
    }

    int step(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st, Prof* pr) override
    {
        b.scal = fb.scal;
        int n = fp64_dt_finalize(DP, fb, 1, st);
        for (int stage = 0; stage < 2; ++stage)
            for (int c = 0; c < kClasses; ++c) {
                const ClassPlan& C = cls[c];
                if (C.doms.empty()) continue;
                const Shape& S = cand[C.best < 0 ? 0 : C.best];
                if (pr) pr->begin("tj_stage3d_mixed", st);
                S.stage(P, class_bufs(c), stage, 0, C.grid, S.smem, st);
                if (pr) pr->end("tj_stage3d_mixed", st);
                n += 1;
            }
        n += fp64_step_end(fb, st);
        return n;
    }

    void describe(char* buf, size_t len) const override
    {
        std::string out;
        for (int c = 0; c < kClasses; ++c) {
            const ClassPlan& C = cls[c];
            if (C.doms.empty()) continue;
            const Shape& S = cand[C.best < 0 ? 0 : C.best];
            char line[192];
            std::snprintf(line, sizeof line, "%s%s boxes (%zu, %lld cells): tile %dx%dx%d, %d tiles, grid %d, smem %zu B",
                          out.empty() ? "" : "; ", kClassName[c], C.doms.size(), C.cells, S.tx, S.ty, S.tz, C.nwork,
                          C.grid, S.smem);
            out += line;
        }
        std::snprintf(buf, len, "%s", out.c_str());
    }
};

}  // namespace

MixedBase* mixed3d_create(const DevParams& DP, const std::vector<DevDomain>& doms, long long ntot, cudaStream_t st,
                          int* err)
{
    auto* m = new Mixed3D();
    *err = m->alloc(DP, doms, ntot, st);
    return m;
}

}  // namespace tj
