// Fused stage kernel of the per-timestep update (2-D fluids), binary32
// (TJ_PRECISION_MIXED) or binary64 (TJ_PRECISION_FUSED64) arithmetic.
//
// One launch per RK stage (HLLCadvance, hllc.cpp:579-695). Each CTA owns a
// 28x28 tile of output cells and does, without leaving the SM:
//   stage : the stage-input primitives of the tile plus a 3-cell halo are
//           staged once in shared memory (ghost cells filled by the boundary
//           mapping of FillDomainBoundary/FillBoundary, main.cpp:124-126);
//   sweep x: one warp per row, one lane per cell. MUSCL (hllc.cpp:541-575),
//           BVD-THINC (thinc.cpp:67-208), cleanUpAlpha, primitiveToConservative
//           and getSoundSpeed of both reconstructed states; the face state of
//           the left neighbour arrives by warp shuffle, the lane computes the
//           HLLC flux of its lower face (hllc.cpp:384-487) and the x update of
//           its cell (hllc.cpp:493-523);
//   sweep y: the same, one warp per column;
//   finish : conservativeToPrimitive (hllc.cpp:689); in the second stage the
//           RK2 average (hllc.cpp:705), cleanUpAlpha (main.cpp:170), the NaN
//           check and the next step's CFL minimum (timestep.cpp:36-70).
// The total energy is stored as a compensated pair (hi + lo) and accumulated
// with an error-free sum; the pressure closure numerator E - KE - sum e_cold
// + sum p_cold, where the cold terms of a stiffened gas cancel E to four
// orders of magnitude, is carried as an unevaluated pair of the working type
// (error-free sums and products, boxaccesscellarray.cpp:116).
// BVD-THINC keeps the reference's scratch history: the alpha of the star
// state of the latest flux sweep (the reference's ULStar), the latest THINC
// right candidate of each cell (URStar, two stamped slots so that a stage
// never reads a value written in the same stage) and the star alpha at box
// hi+1 faces (ULStar's ghost), double-buffered by stage parity.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "tj_math.cuh"
#include "tj_mixed.cuh"

namespace tj {

namespace {

constexpr int MT = 28;           // output tile edge
constexpr int MH = 3;            // staged halo
constexpr int MS = MT + 2 * MH;  // staged cells per axis (34)
constexpr int MP = MS + 1;       // shared-memory pitch (odd: conflict-free columns)
constexpr int CP = MT + 1;       // pitch of the output-cell arrays (odd)
constexpr int NTH = 256;         // threads per CTA
constexpr int NWARP = NTH / 32;
constexpr int XR0 = -2;          // first row (relative to y0) of the x sweep with THINC
constexpr int XRN = 32;          // rows of the x sweep with THINC: y0-2 .. y0+29

// Arithmetic of the working type.
template <typename R>
struct RT;
template <>
struct RT<float> {
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
    static __device__ __forceinline__ float abs_(float a) { return fabsf(a); }
    static __device__ __forceinline__ float sqrt_(float a) { return sqrtf(a); }
    static __device__ __forceinline__ float exp_(float a) { return expf(a); }
    static __device__ __forceinline__ float cosh_(float a) { return coshf(a); }
    static __device__ __forceinline__ float tanh_(float a) { return tanhf(a); }
    static __host__ __device__ constexpr float big() { return 3.0e38f; }
};
template <>
struct RT<double> {
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
    static __device__ __forceinline__ double abs_(double a) { return fabs(a); }
    static __device__ __forceinline__ double sqrt_(double a) { return sqrt(a); }
    static __device__ __forceinline__ double exp_(double a) { return tjm_exp(a); }
    static __device__ __forceinline__ double cosh_(double a) { return tjm_cosh(a); }
    static __device__ __forceinline__ double tanh_(double a) { return tjm_tanh(a); }
    static __host__ __device__ constexpr double big() { return 1.0e300; }
};

template <typename R>
struct MixP {
    int nx, ny, M, thinc;
    int lo_bc[2], hi_bc[2];
    R dx[2], idx[2], beta;
    R mxfloor;  // smallest alpha variation the THINC mixed-cell test accepts (thinc.cpp:86-87: 1e-20)
    R g[TJ_MAX_MAT], ig[TJ_MAX_MAT], pref[TJ_MAX_MAT], eref[TJ_MAX_MAT];
    // pref/Gamma and eref as pairs (hi + lo) for the pressure closure
    R cEh[TJ_MAX_MAT], cEl[TJ_MAX_MAT], eEh[TJ_MAX_MAT], eEl[TJ_MAX_MAT];
    double dxd[2];
    int last_box[4];  // lo x, lo y, hi x, hi y of the last box in MFIter order
};

template <typename R>
struct MixB {
    R* X[2];  // state buffers: 0 = U^n / result, 1 = stage-1 output
    R* starA[2];
    R* gstar[2][2];  // [direction][parity]
    R* urv[2];
    int* urs[2];
    const int* bxlo[2];
    const int* bxhi[2];
    DevScalars* scal;
    int* stage_ctr;
    long long N;
};

// word offsets of the fused state
__host__ __device__ constexpr int W_A(int m) { return m; }
template <int M> __host__ __device__ constexpr int W_AR(int m) { return M + m; }
template <int M> __host__ __device__ constexpr int W_RK(int m) { return 2 * M + m; }
template <int M> __host__ __device__ constexpr int W_RU(int r) { return 3 * M + r; }
template <int M> __host__ __device__ constexpr int W_U(int r) { return 3 * M + 2 + r; }
template <int M> __host__ __device__ constexpr int W_EH() { return 3 * M + 4; }
template <int M> __host__ __device__ constexpr int W_P() { return 3 * M + 5; }
template <int M> __host__ __device__ constexpr int W_EL() { return 3 * M + 6; }
template <int M> __host__ __device__ constexpr int NWORDS() { return 3 * M + 7; }
// staged primitive planes: alpha[M], rho_k[M], u, v, p
template <int M> __host__ __device__ constexpr int NPRIM() { return 2 * M + 3; }

template <typename R, int M>
struct FaceS {
    R a[M], ar[M], rho, ru[2], u[2], E, p, c;
};

// MUSCL slope (hllc.cpp:527-568). With a = u0-um, b = up-u0 and r = a/b, the
// reference's limiter phi(r) = min(2/(1+r), 2r/(1+r)) for r > 0 (0 for r <= 0,
// inf or NaN) applied to (up-um)/2 equals, in exact arithmetic, the argument
// of smaller magnitude when a and b have the same sign and 0 otherwise; the
// fused kernel evaluates that division-free form.
template <typename R>
__device__ __forceinline__ void muscl_f(R um, R u0, R up, R& l, R& r)
{
    const R a = u0 - um, b = up - u0;
    R g = R(0);
    if (a * b > R(0)) g = (RT<R>::abs_(a) < RT<R>::abs_(b)) ? a : b;
    l = u0 - R(0.5) * g;
    r = u0 + R(0.5) * g;
}

// Error-free product of x by a pair (ch + cl): returns hi, adds the rounding
// error and the low-part product to lo.
template <typename R>
__device__ __forceinline__ R two_prod_acc(R ch, R cl, R x, R& lo)
{
    const R p = ch * x;
    lo += RT<R>::fma_(ch, x, -p) + cl * x;
    return p;
}

// Error-free sum: s + e == a + b exactly.
template <typename R>
__device__ __forceinline__ R two_sum(R a, R b, R& e)
{
    const R s = RT<R>::add(a, b);
    const R bb = RT<R>::sub(s, a);
    e = RT<R>::add(RT<R>::sub(a, RT<R>::sub(s, bb)), RT<R>::sub(b, bb));
    return s;
}

// Error-free accumulation of b into a (hi, lo) pair.
template <typename R>
__device__ __forceinline__ void dd_add(R& hi, R& lo, R b)
{
    R e;
    const R s = two_sum<R>(hi, b, e);
    lo = RT<R>::add(lo, e);
    const R t = RT<R>::add(s, lo);
    lo = RT<R>::sub(lo, RT<R>::sub(t, s));
    hi = t;
}

template <typename R, int M>
__device__ __forceinline__ void cleanup_f(R* a)
{
    R tot = R(0);
    int nan = 0;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        R v = a[m];
        if (isnan(v)) {
            v = R(0);
            if (nan == 0) nan = m;
        } else if (v < R(0)) v = R(1e-6);
        else if (v > R(1)) v = R(1);
        a[m] = v;
        tot += v;
    }
    if (nan > 0) {
        a[nan] = R(1) - tot;
        tot += a[nan];
    }
    const R it = R(1) / tot;
#pragma unroll
    for (int m = 0; m < M; ++m) a[m] *= it;
}

// primitiveToConservative + getSoundSpeed of a reconstructed state.
template <typename R, int M>
__device__ __forceinline__ void p2c_f(const MixP<R>& P, const R* rk, FaceS<R, M>& s)
{
    s.rho = R(0);
#pragma unroll
    for (int m = 0; m < M; ++m) {
        s.ar[m] = s.a[m] * rk[m];
        s.rho += s.ar[m];
    }
    R ke = R(0);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        s.ru[r] = s.u[r] * s.rho;
        ke += R(0.5) * s.rho * s.u[r] * s.u[r];
    }
    R G = R(0), ec = R(0), pc = R(0);
#pragma unroll
    for (int m = 0; m < M; ++m) {
        G += s.a[m] * P.ig[m];
        ec += P.eref[m] * s.ar[m];
        pc += P.pref[m] * s.a[m] * P.ig[m];
    }
    s.E = s.p * G + ec - pc + ke;
    R sa = R(0), xt = R(0);
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const R c2 = s.p * (P.g[m] + R(1)) / rk[m] - P.pref[m] / rk[m];
        const R v = P.ig[m] * c2 * s.ar[m] / s.rho;
        sa += (R(0) < v) ? v : R(0);
        xt += P.ig[m] * s.a[m];
    }
    if (sa <= R(0)) sa = R(1e-6);
    s.c = RT<R>::sqrt_(sa / xt);
}

// ---- paired binary32 arithmetic: the two reconstructed states of a cell ----
// A cell's left and right face states (UL, UR) go through the same sequence
// of operations (MUSCL, cleanUpAlpha, primitiveToConservative, getSoundSpeed),
// so the binary32 instance carries them as pairs (x = UL, y = UR) and uses
// Blackwell's paired FFMA2 / FADD2 / FMUL2 instructions: one instruction for
// both states. Every component is rounded as its scalar counterpart would be.
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 f2s(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// fast reciprocal of each component (the -use_fast_math division's)
__device__ __forceinline__ float2 rcp2(float2 a) { return f2(__fdividef(1.0f, a.x), __fdividef(1.0f, a.y)); }

// MUSCL of one primitive: (UL, UR) = u0 -/+ g/2 (muscl_f).
__device__ __forceinline__ float2 muscl_pair(float um, float u0, float up)
{
    const float a = u0 - um, b = up - u0;
    float g = 0.0f;
    if (a * b > 0.0f) g = (fabsf(a) < fabsf(b)) ? a : b;
    return fma2(f2(-0.5f, 0.5f), f2s(g), f2s(u0));
}

// cleanUpAlpha of both states (cleanup_f, componentwise).
template <int M>
__device__ __forceinline__ void cleanup_pair(float2* a)
{
    float2 tot = f2s(0.0f);
    int nanx = 0, nany = 0;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        float vx = a[m].x, vy = a[m].y;
        if (isnan(vx)) { vx = 0.0f; if (nanx == 0) nanx = m; }
        else if (vx < 0.0f) vx = 1e-6f;
        else if (vx > 1.0f) vx = 1.0f;
        if (isnan(vy)) { vy = 0.0f; if (nany == 0) nany = m; }
        else if (vy < 0.0f) vy = 1e-6f;
        else if (vy > 1.0f) vy = 1.0f;
        a[m] = f2(vx, vy);
        tot = add2(tot, a[m]);
    }
    if (nanx > 0) { a[nanx].x = 1.0f - tot.x; tot.x += a[nanx].x; }
    if (nany > 0) { a[nany].y = 1.0f - tot.y; tot.y += a[nany].y; }
    const float2 it = rcp2(tot);
#pragma unroll
    for (int m = 0; m < M; ++m) a[m] = mul2(a[m], it);
}

// primitiveToConservative + getSoundSpeed (p2c_f) of both states, written
// into L (x) and R (y).
template <int M>
__device__ __forceinline__ void p2c_pair(const MixP<float>& P, const float2* a, const float2* rk, const float2* u,
                                         float2 p, FaceS<float, M>& L, FaceS<float, M>& R)
{
    float2 ar[M], rho = f2s(0.0f);
#pragma unroll
    for (int m = 0; m < M; ++m) {
        ar[m] = mul2(a[m], rk[m]);
        rho = add2(rho, ar[m]);
    }
    const float2 hr = mul2(f2s(0.5f), rho);
    float2 ru[2], ke = f2s(0.0f);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        ru[r] = mul2(u[r], rho);
        ke = fma2(mul2(hr, u[r]), u[r], ke);
    }
    float2 G = f2s(0.0f), ec = f2s(0.0f), pc = f2s(0.0f);
#pragma unroll
    for (int m = 0; m < M; ++m) {
        G = fma2(a[m], f2s(P.ig[m]), G);
        ec = fma2(f2s(P.eref[m]), ar[m], ec);
        pc = fma2(mul2(f2s(P.pref[m]), a[m]), f2s(P.ig[m]), pc);
    }
    const float2 E = add2(fma2(p, G, add2(ec, mul2(f2s(-1.0f), pc))), ke);
    const float2 irho = rcp2(rho);
    float2 xt = f2s(0.0f);
    float sax = 0.0f, say = 0.0f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const float2 irk = rcp2(rk[m]);
        const float2 c2 = mul2(fma2(p, f2s(P.g[m] + 1.0f), f2s(-P.pref[m])), irk);
        const float2 v = mul2(mul2(f2s(P.ig[m]), c2), mul2(ar[m], irho));
        sax += (0.0f < v.x) ? v.x : 0.0f;
        say += (0.0f < v.y) ? v.y : 0.0f;
        xt = fma2(f2s(P.ig[m]), a[m], xt);
    }
    if (sax <= 0.0f) sax = 1e-6f;
    if (say <= 0.0f) say = 1e-6f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        L.a[m] = a[m].x;
        R.a[m] = a[m].y;
        L.ar[m] = ar[m].x;
        R.ar[m] = ar[m].y;
    }
    L.rho = rho.x;
    R.rho = rho.y;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        L.ru[r] = ru[r].x;
        R.ru[r] = ru[r].y;
        L.u[r] = u[r].x;
        R.u[r] = u[r].y;
    }
    L.E = E.x;
    R.E = E.y;
    L.p = p.x;
    R.p = p.y;
    L.c = sqrtf(sax / xt.x);
    R.c = sqrtf(say / xt.y);
}

template <typename R, int M>
struct Flux {
    R f[2 * M + 4];  // alpha[M], alphaRho[M], rhoU (2), E; f[2M+3] = S*
};

// HLLC flux of one face (hllc.cpp:384-487); returns the side whose star
// alpha the face carries (0 left, 1 right).
template <typename R, int M>
__device__ __forceinline__ int hllc_f(const FaceS<R, M>& L, const FaceS<R, M>& Rt, int d, Flux<R, M>& F)
{
    const R x1 = RT<R>::abs_(L.u[d]) + L.c, x2 = RT<R>::abs_(Rt.u[d]) + Rt.c;
    const R SR = (x1 < x2) ? x2 : x1;
    const R SL = -SR;
    const R Ss = (Rt.p - L.p + L.ru[d] * (SL - L.u[d]) - Rt.ru[d] * (SR - Rt.u[d])) /
                 (L.rho * (SL - L.u[d]) - Rt.rho * (SR - Rt.u[d]));
    F.f[2 * M + 3] = Ss;
    const bool left = (SL >= R(0)) || (Ss >= R(0));
    const bool hllc = left ? !(SL >= R(0)) : (SR >= R(0));
    const FaceS<R, M>& K = left ? L : Rt;
    const R SK = left ? SL : SR;
    const R uK = K.u[d];
    const R mult = (RT<R>::abs_((Ss - uK) / Ss) < R(1e-20)) ? R(1) : (SK - uK) / (SK - Ss);
    R rs = R(0), ars[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        ars[m] = mult * K.ar[m];
        rs += ars[m];
    }
    R rus[2];
    rus[d] = mult * K.rho * Ss;
    rus[1 - d] = mult * K.ru[1 - d];
    const R usd = rus[d] / rs;
    const R Es = mult * K.rho * (K.E / K.rho + (Ss - uK) * (Ss + K.p / (K.rho * (SK - uK))));
    const R w = hllc ? SK : R(0);
#pragma unroll
    for (int m = 0; m < M; ++m) {
        F.f[m] = K.a[m] * usd;
        F.f[M + m] = K.ar[m] * uK + w * (ars[m] - K.ar[m]);
    }
    F.f[2 * M + d] = K.ru[d] * uK + K.p + w * (rus[d] - K.ru[d]);
    F.f[2 * M + 1 - d] = K.ru[1 - d] * uK + w * (rus[1 - d] - K.ru[1 - d]);
    F.f[2 * M + 2] = (K.E + K.p) * uK + w * (Es - K.E);
    return left ? 0 : 1;
}

template <typename R>
struct Cand {
    unsigned mask;
    R L[TJ_MAX_MAT], Rr[TJ_MAX_MAT];
};

// Boundary image of index i (foextrap: nearest cell; reflect: mirror). Images
// deeper than the domain is wide are clamped into it; only ghost depths up to
// two are ever consumed.
__device__ __forceinline__ int reflect_map(int i, int n, int lo_bc, int hi_bc, bool& refl)
{
    refl = false;
    int j = i;
    if (i < 0) {
        if (lo_bc == TJ_BC_REFLECTIVE) { refl = true; j = -1 - i; }
        else j = 0;
    } else if (i > n - 1) {
        if (hi_bc == TJ_BC_REFLECTIVE) { refl = true; j = 2 * n - 1 - i; }
        else j = n - 1;
    }
    return j < 0 ? 0 : (j > n - 1 ? n - 1 : j);
}

template <typename R>
__device__ __forceinline__ R ur_read(const MixB<R>& b, int m, long long c, int s)
{
    const long long k = (long long)m * b.N + c;
    const int s0 = b.urs[0][k], s1 = b.urs[1][k];
    R v = R(0);
    int best = -1;
    if (s0 < s && s0 > best) { best = s0; v = b.urv[0][k]; }
    if (s1 < s && s1 > best) { v = b.urv[1][k]; }
    return v;
}

template <typename R>
__device__ __forceinline__ void ur_write(const MixB<R>& b, int m, long long c, int s, R v)
{
    const long long k = (long long)m * b.N + c;
    const int slot = (b.urs[0][k] <= b.urs[1][k]) ? 0 : 1;
    b.urv[slot][k] = v;
    b.urs[slot][k] = s;
}

// Shared-memory layout of one CTA (in words of the working type).
template <typename R, int M, bool THINC>
struct Smem {
    static constexpr int NP = NPRIM<M>();
    static constexpr int NC = 2 * M + 4;  // alpha[M], alphaRho[M], rhoU(2), E hi, E lo
    static constexpr int U_OFF = 0;
    static constexpr int CT = MT * CP;  // one output-cell plane
    static constexpr int C_OFF = U_OFF + NP * MS * MP;
    static constexpr int SAX_OFF = C_OFF + NC * CT;                      // star alpha of x faces, rows y0-1..y0+29
    static constexpr int CRX_OFF = SAX_OFF + (THINC ? M * 31 * CP : 0);  // x right candidates, rows y0-2..y0+28
    static constexpr int RED_OFF = CRX_OFF + (THINC ? M * 31 * CP : 0);
    static constexpr int TOTAL = RED_OFF + 32;
    // x mixed masks, one byte per cell (rows y0-2..y0+28), after the words
    static constexpr int MXB = THINC ? 31 * CP : 0;
    // 74.6 KB for binary32, M = 2, THINC: three CTAs fit on an SM; the star
    // alpha of the y faces and the new URStar values go straight to global
    // memory from the y sweep instead of through shared memory
    static constexpr size_t BYTES = sizeof(R) * TOTAL + ((MXB + 15) / 16) * 16;
};

// The THINC candidate of the cell at staged position (tx, ty) along d.
template <typename R, int M>
__device__ __forceinline__ void thinc_cand_f(const MixP<R>& P, const R* sU, int tx, int ty, int d, Cand<R>& c)
{
    const int ox = d == 0 ? 1 : 0, oy = d == 0 ? 0 : 1;
    c.mask = 0;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const R* A = sU + m * MS * MP;
        const R aL = A[(ty - oy) * MP + tx - ox], aR = A[(ty + oy) * MP + tx + ox], a0 = A[ty * MP + tx];
        const R mn = (aR < aL) ? aR : aL;
        const R mx = ((aL < aR) ? aR : aL) - mn;
        const R theta = (R)((R(0) < aR - aL) - (aR - aL < R(0)));
        // C = (a0-mn+eps)/(mx+eps) (0 when mx < eps); the interval test is
        // made on the numerator so that the division is only done when mixed
        const R num = a0 - mn + R(1e-20), den = mx + R(1e-20);
        const bool mixed = !(mx < P.mxfloor) && (num > R(1e-4) * den) && (num < (R(0.999999) - R(1e-4)) * den) &&
                           ((aR - a0) * (a0 - aL) >= R(0));
        c.L[m] = R(0);
        c.Rr[m] = R(0);
        if (mixed) {
            const R C = num / den;
            c.mask |= 1u << m;
            const R nx = -R(1) / (R(8) * P.dx[0]) *
                         (A[(ty + 1) * MP + tx + 1] + R(2) * A[ty * MP + tx + 1] + A[(ty - 1) * MP + tx + 1] -
                          A[(ty + 1) * MP + tx - 1] - R(2) * A[ty * MP + tx - 1] - A[(ty - 1) * MP + tx - 1]);
            const R ny = -R(1) / (R(8) * P.dx[1]) *
                         (A[(ty + 1) * MP + tx + 1] + R(2) * A[(ty + 1) * MP + tx] + A[(ty + 1) * MP + tx - 1] -
                          A[(ty - 1) * MP + tx - 1] - R(2) * A[(ty - 1) * MP + tx] - A[(ty - 1) * MP + tx + 1]);
            const R norm = RT<R>::sqrt_(nx * nx + ny * ny);
            const R nvc = (norm < R(1e-20)) ? R(0) : RT<R>::abs_((d == 0 ? nx : ny) / norm);
            const R beta = nvc * P.beta + R(0.01);
            const R coshB = RT<R>::cosh_(beta), tanhB = RT<R>::tanh_(beta);
            const R B = RT<R>::exp_(theta * beta * ((R(2) * C) - R(1)));
            const R Aa = ((B / coshB) - R(1)) / tanhB;
            c.Rr[m] = mn + (mx / R(2)) * (R(1) + theta * ((tanhB + Aa) / (R(1) + Aa * tanhB)));
            c.L[m] = mn + (mx / R(2)) * (R(1) + theta * Aa);
        }
    }
}

// Asynchronous global -> shared copy of one word (cp.async, 4 or 8 bytes).
template <typename R>
__device__ __forceinline__ void cp_async_r(R* dst, const R* src)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(R) == 4) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(a), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(a), "l"(src) : "memory");
}

// One sweep line (a row for D = 0, a column for D = 1) of 32 lanes.
template <typename R, int M, bool THINC, int D>
__device__ void sweep_line(const MixP<R>& P, const MixB<R>& b, R* sm, int x0, int y0, int line, int s, R dtdx,
                           bool want_flux)
{
    using SM = Smem<R, M, THINC>;
    const R* sU = sm + SM::U_OFF;
    const int lane = threadIdx.x & 31;
    const int n = D == 0 ? P.nx : P.ny;
    const int p0 = (D == 0 ? x0 : y0) - 2;
    const int pos = p0 + lane;  // cell position along d
    // staged coordinates of this lane's cell
    const int tx = D == 0 ? lane + 1 : line - x0 + MH;
    const int ty = D == 0 ? line - y0 + MH : lane + 1;
    const int ox = D == 0 ? 1 : 0, oy = D == 0 ? 0 : 1;
    constexpr int NP = NPRIM<M>();
    R ul[NP], ur[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        const R* Q = sU + q * MS * MP;
        const R um = Q[(ty - oy) * MP + tx - ox], u0 = Q[ty * MP + tx], up = Q[(ty + oy) * MP + tx + ox];
        if constexpr (sizeof(R) == 4) {
            const float2 lr = muscl_pair(um, u0, up);
            ul[q] = lr.x;
            ur[q] = lr.y;
        } else {
            muscl_f<R>(um, u0, up, ul[q], ur[q]);
        }
    }
    // ---- BVD-THINC (thinc.cpp:67-208) ----
    Cand<R> cd;
    cd.mask = 0;
    const bool valid = pos >= 0 && pos < n;
    if (THINC) thinc_cand_f<R, M>(P, sU, tx, ty, D, cd);
    const bool flag = THINC && ((cd.mask >> (M - 1)) & 1u);
    // the TBV comparison only runs in lines that hold a flagged cell
    if (THINC && __any_sync(0xffffffffu, flag && valid && lane >= 1 && lane <= 30)) {
        const unsigned mm = __shfl_up_sync(0xffffffffu, cd.mask, 1), mp = __shfl_down_sync(0xffffffffu, cd.mask, 1);
        const int lo = valid ? b.bxlo[D][pos] : 0, hi = valid ? b.bxhi[D][pos] : -1;
        const bool in_m = valid && pos - 1 >= lo, in_p = valid && pos + 1 <= hi;
        const int cx = D == 0 ? pos : line, cy = D == 0 ? line : pos;
        const long long cell = cx + (long long)P.nx * cy;
        const int par_in = (s + 1) & 1;
        const bool need = flag && valid && lane >= 1 && lane <= 30;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const R urm_m = __shfl_up_sync(0xffffffffu, ur[m], 1);    // MUSCL UR alpha of pos-1
            const R ulp_m = __shfl_down_sync(0xffffffffu, ul[m], 1);  // MUSCL UL alpha of pos+1
            const R cRm = __shfl_up_sync(0xffffffffu, cd.Rr[m], 1);
            const R cLp = __shfl_down_sync(0xffffffffu, cd.L[m], 1);
            if (!need) continue;
            const R* A = sU + m * MS * MP;
            R urm, ulp, trm, tlp;
            if (in_m) {
                urm = urm_m;
                if ((mm >> m) & 1u) trm = cRm;
                else if (D == 0) trm = ur_read<R>(b, m, cell - 1, s);  // URStar before this sweep
                else {
                    const int r = pos - 1 - (y0 - 2);
                    const unsigned mx = reinterpret_cast<const unsigned char*>(sm + SM::TOTAL)[r * CP + (line - x0)];
                    trm = ((mx >> m) & 1u) ? sm[SM::CRX_OFF + (m * 31 + r) * CP + (line - x0)]
                                           : ur_read<R>(b, m, cell - P.nx, s);
                }
            } else {
                urm = A[(ty - oy) * MP + tx - ox];
                trm = R(0);  // URStar ghosts are never written
            }
            if (in_p) {
                ulp = ulp_m;
                if ((mp >> m) & 1u) tlp = cLp;
                else if (D == 0) tlp = b.starA[par_in][(long long)m * b.N + cell + 1];
                else tlp = sm[SM::SAX_OFF + (m * 31 + (pos + 1 - (y0 - 1))) * CP + (line - x0)];
            } else {
                ulp = A[(ty + oy) * MP + tx + ox];
                const long long nfd = D == 0 ? (long long)(P.nx + 1) * P.ny : (long long)P.nx * (P.ny + 1);
                const long long f = D == 0 ? (pos + 1) + (long long)(P.nx + 1) * line : line + (long long)P.nx * (pos + 1);
                tlp = b.gstar[D][par_in][(long long)m * nfd + f];
            }
            R tpl, tpr;
            if ((cd.mask >> m) & 1u) {
                tpl = cd.L[m];
                tpr = cd.Rr[m];
            } else if (D == 0) {
                tpl = b.starA[par_in][(long long)m * b.N + cell];
                tpr = ur_read<R>(b, m, cell, s);
            } else {
                const int r = pos - (y0 - 2);
                const unsigned mx = reinterpret_cast<const unsigned char*>(sm + SM::TOTAL)[r * CP + (line - x0)];
                tpl = sm[SM::SAX_OFF + (m * 31 + (pos - (y0 - 1))) * CP + (line - x0)];
                tpr = ((mx >> m) & 1u) ? sm[SM::CRX_OFF + (m * 31 + r) * CP + (line - x0)] : ur_read<R>(b, m, cell, s);
            }
            const R upl = ul[m], upr = ur[m];
#define MNF(a_, b_) (((b_) < (a_)) ? (b_) : (a_))
#define ABSR(x_) RT<R>::abs_(x_)
#define TBVF(PL, PR) \
    MNF(MNF(ABSR(urm - (PL)) + ABSR((PR)-ulp), ABSR(trm - (PL)) + ABSR((PR)-tlp)), \
        MNF(ABSR(urm - (PL)) + ABSR((PR)-tlp), ABSR(trm - (PL)) + ABSR((PR)-ulp)))
            const R tm_ = TBVF(upl, upr), tt_ = TBVF(tpl, tpr);
#undef TBVF
#undef ABSR
#undef MNF
            if (tt_ < tm_) {
                ul[m] = tpl;
                ur[m] = tpr;
            }
        }
    }
    // ---- cleanUpAlpha, primitiveToConservative, getSoundSpeed ----
    FaceS<R, M> SLs, SRs;
    if constexpr (sizeof(R) == 4) {
        float2 a2[M], rk2[M], u2[2];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            a2[m] = f2(ul[m], ur[m]);
            rk2[m] = f2(ul[M + m], ur[M + m]);
        }
        if (THINC) cleanup_pair<M>(a2);
#pragma unroll
        for (int r = 0; r < 2; ++r) u2[r] = f2(ul[2 * M + r], ur[2 * M + r]);
        p2c_pair<M>(P, a2, rk2, u2, f2(ul[2 * M + 2], ur[2 * M + 2]), SLs, SRs);
    } else {
        R rkl[M], rkr[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            SLs.a[m] = ul[m];
            SRs.a[m] = ur[m];
            rkl[m] = ul[M + m];
            rkr[m] = ur[M + m];
        }
        if (THINC) {
            cleanup_f<R, M>(SLs.a);
            cleanup_f<R, M>(SRs.a);
        }
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            SLs.u[r] = ul[2 * M + r];
            SRs.u[r] = ur[2 * M + r];
        }
        SLs.p = ul[2 * M + 2];
        SRs.p = ur[2 * M + 2];
        p2c_f<R, M>(P, rkl, SLs);
        p2c_f<R, M>(P, rkr, SRs);
    }

    // ---- ghost lanes take the boundary image of a valid lane's state ----
    if (p0 < 0 || p0 + 31 >= n) {  // only lines that reach the domain boundary
        bool refl;
        const int src = reflect_map(pos, n, P.lo_bc[D], P.hi_bc[D], refl);
        const int src_lane = src - p0;
        const int sl = (src_lane >= 0 && src_lane < 32) ? src_lane : lane;
        FaceS<R, M>* S2[2] = {&SLs, &SRs};
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            FaceS<R, M>& S = *S2[side];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                S.a[m] = __shfl_sync(0xffffffffu, S.a[m], sl);
                S.ar[m] = __shfl_sync(0xffffffffu, S.ar[m], sl);
            }
            S.rho = __shfl_sync(0xffffffffu, S.rho, sl);
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                S.ru[r] = __shfl_sync(0xffffffffu, S.ru[r], sl);
                S.u[r] = __shfl_sync(0xffffffffu, S.u[r], sl);
            }
            S.E = __shfl_sync(0xffffffffu, S.E, sl);
            S.p = __shfl_sync(0xffffffffu, S.p, sl);
            S.c = __shfl_sync(0xffffffffu, S.c, sl);
            if (refl) {
                S.u[D] = -S.u[D];
                S.ru[D] = -S.ru[D];
            }
        }
    }
    const bool out_cell = lane >= 2 && lane <= 29 && valid;
    if (THINC && D == 0) {
        // x candidates needed by the y sweep (URStar before the y sweep)
        const int r = line - (y0 - 2);
        if (r >= 0 && r < 31 && out_cell) {
            reinterpret_cast<unsigned char*>(sm + SM::TOTAL)[r * CP + (pos - x0)] = (unsigned char)cd.mask;
#pragma unroll
            for (int m = 0; m < M; ++m) sm[SM::CRX_OFF + (m * 31 + r) * CP + (pos - x0)] = cd.Rr[m];
        }
    }
    if (!want_flux) return;

    // ---- flux of the lower face: left state UR of pos-1, right state UL of pos ----
    FaceS<R, M> Lf;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        Lf.a[m] = __shfl_up_sync(0xffffffffu, SRs.a[m], 1);
        Lf.ar[m] = __shfl_up_sync(0xffffffffu, SRs.ar[m], 1);
    }
    Lf.rho = __shfl_up_sync(0xffffffffu, SRs.rho, 1);
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        Lf.ru[r] = __shfl_up_sync(0xffffffffu, SRs.ru[r], 1);
        Lf.u[r] = __shfl_up_sync(0xffffffffu, SRs.u[r], 1);
    }
    Lf.E = __shfl_up_sync(0xffffffffu, SRs.E, 1);
    Lf.p = __shfl_up_sync(0xffffffffu, SRs.p, 1);
    Lf.c = __shfl_up_sync(0xffffffffu, SRs.c, 1);
    Flux<R, M> F;
    const int side = hllc_f<R, M>(Lf, SLs, D, F);
    R astar[M];
#pragma unroll
    for (int m = 0; m < M; ++m) astar[m] = side ? SLs.a[m] : Lf.a[m];

    // the face is owned by this tile if its right cell is an output cell, or
    // if it is the domain's hi face and its left cell is an output cell
    const bool hi_face = pos == n && lane >= 3 && lane <= 30;
    if (THINC) {
        // star alpha: x faces kept in shared memory (rows y0-1..y0+29) for
        // the y sweep; the y faces of output cells (the next stage's ULStar)
        // take their cell's place in the same array: each y-sweep warp reads
        // only its own column of it, and all its reads come before this write
        if (D == 0 || out_cell) {
            const int r = D == 0 ? line - (y0 - 1) : pos - (y0 - 1);
            const int col = D == 0 ? pos - x0 : line - x0;
            if (r >= 0 && r < 31 && out_cell)
#pragma unroll
                for (int m = 0; m < M; ++m) sm[SM::SAX_OFF + (m * 31 + r) * CP + col] = astar[m];
        }
        // ULStar ghost at the hi+1 face of the box to the face's left
        const bool line_out = D == 0 ? (line >= y0 && line < y0 + MT && line < P.ny) : true;
        if ((out_cell || hi_face) && line_out && pos >= 1 && b.bxhi[D][pos - 1] == pos - 1) {
            const int par_out = s & 1;
            const long long nfd = D == 0 ? (long long)(P.nx + 1) * P.ny : (long long)P.nx * (P.ny + 1);
            const long long f = D == 0 ? pos + (long long)(P.nx + 1) * line : line + (long long)P.nx * pos;
#pragma unroll
            for (int m = 0; m < M; ++m) b.gstar[D][par_out][(long long)m * nfd + f] = astar[m];
        }
        if (D == 1 && out_cell) {
            // the cell's URStar after this stage: y candidate, else x candidate
            // (versioned by stage: readers of this stage see the previous value)
            const int r = pos - (y0 - 2);
            const unsigned mxm = reinterpret_cast<const unsigned char*>(sm + SM::TOTAL)[r * CP + (line - x0)];
            const unsigned f = cd.mask | mxm;
            if (f) {
                const long long cell = line + (long long)P.nx * pos;
#pragma unroll
                for (int m = 0; m < M; ++m)
                    if ((f >> m) & 1u)
                        ur_write<R>(b, m, cell, s,
                                    ((cd.mask >> m) & 1u) ? cd.Rr[m] : sm[SM::CRX_OFF + (m * 31 + r) * CP + (line - x0)]);
            }
        }
    }

    // ---- update of the lane's cell: needs the flux of the upper face ----
    R fu[2 * M + 4];
#pragma unroll
    for (int q = 0; q < 2 * M + 4; ++q) fu[q] = __shfl_down_sync(0xffffffffu, F.f[q], 1);
    const bool upd_line = D == 0 ? (line >= y0 && line < y0 + MT && line < P.ny) : true;
    if (!(out_cell && upd_line)) return;
    const int ci = D == 0 ? pos - x0 : line - x0;  // output tile column
    const int cj = D == 0 ? line - y0 : pos - y0;  // output tile row
    R* C = sm + SM::C_OFF;
    const int oc = cj * CP + ci;
    constexpr int MTT = SM::CT;
    const R dS = F.f[2 * M + 3] - fu[2 * M + 3];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const R a0 = sU[m * MS * MP + ty * MP + tx];
        C[m * MTT + oc] += dtdx * (F.f[m] - fu[m] - a0 * dS);
        C[(M + m) * MTT + oc] += dtdx * (F.f[M + m] - fu[M + m]);
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) C[(2 * M + r) * MTT + oc] += dtdx * (F.f[2 * M + r] - fu[2 * M + r]);
    R eh = C[(2 * M + 2) * MTT + oc], el = C[(2 * M + 3) * MTT + oc];
    dd_add<R>(eh, el, dtdx * (F.f[2 * M + 2] - fu[2 * M + 2]));
    C[(2 * M + 2) * MTT + oc] = eh;
    C[(2 * M + 3) * MTT + oc] = el;
}

template <typename R, int M, bool THINC>
__global__ void __launch_bounds__(NTH, sizeof(R) == 4 ? 3 : 1) k_stage2d(MixP<R> P, MixB<R> b, int stage)
{
    if (b.scal->done) return;
    using SM = Smem<R, M, THINC>;
    extern __shared__ __align__(16) unsigned char smraw[];
    R* sm = reinterpret_cast<R*>(smraw);
    const int x0 = blockIdx.x * MT, y0 = blockIdx.y * MT;
    const int s = *b.stage_ctr + stage;
    const R* __restrict__ Xin = b.X[stage];
    R* __restrict__ Xout = b.X[stage == 0 ? 1 : 0];
    const long long N = b.N;
    // binary32: dt/dx as a product with 1/dx (no binary64 division per thread)
    const R dtdx = sizeof(R) == 8 ? (R)(b.scal->dt / P.dxd[0]) : (R)b.scal->dt * P.idx[0];
    const R dtdy = sizeof(R) == 8 ? (R)(b.scal->dt / P.dxd[1]) : (R)b.scal->dt * P.idx[1];

    // ---- stage the primitives of tile + halo and the output cells' conserved
    //      words (U1 = U, hllc.cpp:583) with asynchronous copies: every copy is
    //      in flight at once, none holds a register ----
    for (int t = threadIdx.x; t < MS * MS; t += NTH) {
        const int tx = t % MS, ty = t / MS;
        bool rx, ry;
        const int gx = reflect_map(x0 - MH + tx, P.nx, P.lo_bc[0], P.hi_bc[0], rx);
        const int gy = reflect_map(y0 - MH + ty, P.ny, P.lo_bc[1], P.hi_bc[1], ry);
        const long long g = gx + (long long)P.nx * gy;
        R* Su = sm + SM::U_OFF + ty * MP + tx;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            cp_async_r(Su + m * MS * MP, Xin + W_A(m) * N + g);
            cp_async_r(Su + (M + m) * MS * MP, Xin + W_RK<M>(m) * N + g);
        }
        cp_async_r(Su + (2 * M) * MS * MP, Xin + W_U<M>(0) * N + g);
        cp_async_r(Su + (2 * M + 1) * MS * MP, Xin + W_U<M>(1) * N + g);
        cp_async_r(Su + (2 * M + 2) * MS * MP, Xin + W_P<M>() * N + g);
    }
    for (int t = threadIdx.x; t < MT * MT; t += NTH) {
        const int ci = t % MT, cj = t / MT;
        const int gx = x0 + ci, gy = y0 + cj;
        if (gx >= P.nx || gy >= P.ny) continue;
        const long long g = gx + (long long)P.nx * gy;
        R* Sc = sm + SM::C_OFF + cj * CP + ci;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            cp_async_r(Sc + m * SM::CT, Xin + W_A(m) * N + g);
            cp_async_r(Sc + (M + m) * SM::CT, Xin + W_AR<M>(m) * N + g);
        }
        cp_async_r(Sc + (2 * M) * SM::CT, Xin + W_RU<M>(0) * N + g);
        cp_async_r(Sc + (2 * M + 1) * SM::CT, Xin + W_RU<M>(1) * N + g);
        cp_async_r(Sc + (2 * M + 2) * SM::CT, Xin + W_EH<M>() * N + g);
        cp_async_r(Sc + (2 * M + 3) * SM::CT, Xin + W_EL<M>() * N + g);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    if (stage == 1) {
        // The second stage's finish averages with U^n (hllc.cpp:705), which
        // the first stage's output has mostly pushed out of L2: ask for the
        // output cells' rows of every U^n word now, so that they arrive
        // while the sweeps run (both ends of each 28-cell row, which may
        // span two 128-byte lines).
        constexpr int NW = NWORDS<M>();
        for (int t = threadIdx.x; t < NW * MT * 2; t += NTH) {
            const int w = t / (2 * MT), r = (t >> 1) % MT, e = t & 1;
            const int gx = min(x0 + e * (MT - 1), P.nx - 1), gy = y0 + r;
            if (gy < P.ny) {
                const R* a = Xout + (long long)w * N + gx + (long long)P.nx * gy;
                asm volatile("prefetch.global.L2 [%0];\n" ::"l"(a));
            }
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
    // reflect_odd ghosts (FillDomainBoundary): negate the normal velocity of
    // staged cells that mirror across a reflective face
    if ((P.lo_bc[0] == TJ_BC_REFLECTIVE && x0 < MH) || (P.hi_bc[0] == TJ_BC_REFLECTIVE && x0 - MH + MS > P.nx) ||
        (P.lo_bc[1] == TJ_BC_REFLECTIVE && y0 < MH) || (P.hi_bc[1] == TJ_BC_REFLECTIVE && y0 - MH + MS > P.ny)) {
        for (int t = threadIdx.x; t < MS * MS; t += NTH) {
            const int tx = t % MS, ty = t / MS;
            bool rx, ry;
            reflect_map(x0 - MH + tx, P.nx, P.lo_bc[0], P.hi_bc[0], rx);
            reflect_map(y0 - MH + ty, P.ny, P.lo_bc[1], P.hi_bc[1], ry);
            R* Su = sm + SM::U_OFF + ty * MP + tx;
            if (rx) Su[(2 * M) * MS * MP] = -Su[(2 * M) * MS * MP];
            if (ry) Su[(2 * M + 1) * MS * MP] = -Su[(2 * M + 1) * MS * MP];
        }
        __syncthreads();
    }

    const int warp = threadIdx.x >> 5;
    // ---- x sweep: rows ----
    {
        const int r0 = THINC ? y0 + XR0 : y0;
        const int nr = THINC ? XRN : MT;
        for (int r = warp; r < nr; r += NWARP) {
            const int line = r0 + r;
            if (line < 0 || line >= P.ny) continue;
            sweep_line<R, M, THINC, 0>(P, b, sm, x0, y0, line, s, dtdx, !THINC || line >= y0 - 1);
        }
    }
    __syncthreads();
    // ---- y sweep: columns ----
    for (int c = warp; c < MT; c += NWARP) {
        const int line = x0 + c;
        if (line >= P.nx) continue;
        sweep_line<R, M, THINC, 1>(P, b, sm, x0, y0, line, s, dtdy, true);
    }
    __syncthreads();

    // ---- finish: c2p; stage 2: average, cleanUpAlpha, CFL, NaN check ----
    R dtmin = RT<R>::big();
    bool nan_seen = false;
    for (int t = threadIdx.x; t < MT * MT; t += NTH) {
        const int ci = t % MT, cj = t / MT;
        const int gx = x0 + ci, gy = y0 + cj;
        if (gx >= P.nx || gy >= P.ny) continue;
        const long long g = gx + (long long)P.nx * gy;
        const int oc = cj * CP + ci;
        R a[M], ar[M], rk[M], ru[2], u[2], eh, el, p;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            a[m] = sm[SM::C_OFF + m * SM::CT + oc];
            ar[m] = sm[SM::C_OFF + (M + m) * SM::CT + oc];
        }
        ru[0] = sm[SM::C_OFF + (2 * M) * SM::CT + oc];
        ru[1] = sm[SM::C_OFF + (2 * M + 1) * SM::CT + oc];
        eh = sm[SM::C_OFF + (2 * M + 2) * SM::CT + oc];
        el = sm[SM::C_OFF + (2 * M + 3) * SM::CT + oc];
        // conservativeToPrimitive (boxaccesscellarray.cpp:67-122)
        R rho = R(0);
#pragma unroll
        for (int m = 0; m < M; ++m) {
            rk[m] = ar[m] / a[m];
            rho += ar[m];
        }
        R ke = R(0);
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            u[r] = ru[r] / rho;
            ke += R(0.5) * rho * u[r] * u[r];
        }
        // p = (E - KE - sum e_cold + sum p_cold) / sum alpha/Gamma
        // (boxaccesscellarray.cpp:116), numerator as an unevaluated pair
        R sh = eh, sl = el, e, lo;
        sh = two_sum<R>(sh, -ke, e);
        sl += e;
        R G = R(0);
#pragma unroll
        for (int m = 0; m < M; ++m) {
            lo = R(0);
            const R ec = two_prod_acc<R>(P.eEh[m], P.eEl[m], ar[m], lo);
            sh = two_sum<R>(sh, -ec, e);
            sl += e - lo;
            lo = R(0);
            const R pc = two_prod_acc<R>(P.cEh[m], P.cEl[m], a[m], lo);
            sh = two_sum<R>(sh, pc, e);
            sl += e + lo;
            G += a[m] * P.ig[m];
        }
        p = (sh + sl) / G;
        if (stage == 1) {
            // U1 = U*0.5 + U2*0.5 over the carried state (hllc.cpp:705)
#pragma unroll
            for (int m = 0; m < M; ++m) {
                a[m] = R(0.5) * Xout[W_A(m) * N + g] + R(0.5) * a[m];
                ar[m] = R(0.5) * Xout[W_AR<M>(m) * N + g] + R(0.5) * ar[m];
                rk[m] = R(0.5) * Xout[W_RK<M>(m) * N + g] + R(0.5) * rk[m];
            }
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                ru[r] = R(0.5) * Xout[W_RU<M>(r) * N + g] + R(0.5) * ru[r];
                u[r] = R(0.5) * Xout[W_U<M>(r) * N + g] + R(0.5) * u[r];
            }
            p = R(0.5) * Xout[W_P<M>() * N + g] + R(0.5) * p;
            R hs = R(0.5) * Xout[W_EH<M>() * N + g], ls = R(0.5) * Xout[W_EL<M>() * N + g];
            dd_add<R>(hs, ls, R(0.5) * eh);
            ls = RT<R>::add(ls, R(0.5) * el);
            const R tt = RT<R>::add(hs, ls);
            el = RT<R>::sub(ls, RT<R>::sub(tt, hs));
            eh = tt;
            cleanup_f<R, M>(a);  // main.cpp:170
            // next step's CFL (timestep.cpp:7-29), rho = sum alphaRho
            R rr = R(0), sa = R(0), xt = R(0);
#pragma unroll
            for (int m = 0; m < M; ++m) rr += ar[m];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const R c2 = p * (P.g[m] + R(1)) / rk[m] - P.pref[m] / rk[m];
                const R v = P.ig[m] * c2 * ar[m] / rr;
                sa += (R(0) < v) ? v : R(0);
                xt += P.ig[m] * a[m];
            }
            if (sa <= R(0)) sa = R(1e-6);
            const R cs = RT<R>::sqrt_(sa / xt);
            const R v0 = P.dx[0] / (cs + RT<R>::abs_(u[0])), v1 = P.dx[1] / (cs + RT<R>::abs_(u[1]));
            if (v0 < dtmin) dtmin = v0;
            if (v1 < dtmin) dtmin = v1;
            if (gx >= P.last_box[0] && gx <= P.last_box[2] && gy >= P.last_box[1] && gy <= P.last_box[3]) {
                bool nn = isnan(eh) || isnan(p);
#pragma unroll
                for (int m = 0; m < M; ++m) nn |= isnan(a[m]) || isnan(ar[m]) || isnan(rk[m]);
                nn |= isnan(ru[0]) || isnan(ru[1]) || isnan(u[0]) || isnan(u[1]);
                nan_seen |= nn;
            }
        }
#pragma unroll
        for (int m = 0; m < M; ++m) {
            Xout[W_A(m) * N + g] = a[m];
            Xout[W_AR<M>(m) * N + g] = ar[m];
            Xout[W_RK<M>(m) * N + g] = rk[m];
        }
        Xout[W_RU<M>(0) * N + g] = ru[0];
        Xout[W_RU<M>(1) * N + g] = ru[1];
        Xout[W_U<M>(0) * N + g] = u[0];
        Xout[W_U<M>(1) * N + g] = u[1];
        Xout[W_EH<M>() * N + g] = eh;
        Xout[W_EL<M>() * N + g] = el;
        Xout[W_P<M>() * N + g] = p;
        if (THINC)
#pragma unroll
            for (int m = 0; m < M; ++m)
                b.starA[s & 1][(long long)m * N + g] = sm[SM::SAX_OFF + (m * 31 + (cj + 1)) * CP + ci];
    }
    if (stage == 1) {
        if (nan_seen) atomicOr(&b.scal->nan_flag, 1);
        for (int o = 16; o > 0; o >>= 1) {
            const R w = __shfl_down_sync(0xffffffffu, dtmin, o);
            dtmin = (w < dtmin) ? w : dtmin;
        }
        R* red = sm + SM::RED_OFF;
        const int lane = threadIdx.x & 31;
        __syncthreads();
        if (lane == 0) red[warp] = dtmin;
        __syncthreads();
        if (threadIdx.x == 0) {
            R mn = red[0];
            for (int w = 1; w < NWARP; ++w) mn = (red[w] < mn) ? red[w] : mn;
            atomicMin(&b.scal->dtmin_bits, (unsigned long long)__double_as_longlong((double)mn));
        }
    }
}

// CFL of the current state (used after the state is set from outside).
template <typename R, int M>
__global__ void k_cfl_mixed(MixP<R> P, MixB<R> b)
{
    R dtmin = RT<R>::big();
    const long long N = b.N;
    const R* X = b.X[0];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        R rr = R(0), sa = R(0), xt = R(0), ar[M], a[M], rk[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            a[m] = X[W_A(m) * N + g];
            ar[m] = X[W_AR<M>(m) * N + g];
            rk[m] = X[W_RK<M>(m) * N + g];
            rr += ar[m];
        }
        const R p = X[W_P<M>() * N + g];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            const R c2 = p * (P.g[m] + R(1)) / rk[m] - P.pref[m] / rk[m];
            const R v = P.ig[m] * c2 * ar[m] / rr;
            sa += (R(0) < v) ? v : R(0);
            xt += P.ig[m] * a[m];
        }
        if (sa <= R(0)) sa = R(1e-6);
        const R cs = RT<R>::sqrt_(sa / xt);
        const R v0 = P.dx[0] / (cs + RT<R>::abs_(X[W_U<M>(0) * N + g]));
        const R v1 = P.dx[1] / (cs + RT<R>::abs_(X[W_U<M>(1) * N + g]));
        if (v0 < dtmin) dtmin = v0;
        if (v1 < dtmin) dtmin = v1;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const R w = __shfl_down_sync(0xffffffffu, dtmin, o);
        dtmin = (w < dtmin) ? w : dtmin;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(&b.scal->dtmin_bits, (unsigned long long)__double_as_longlong((double)dtmin));
}

// FP64 carried state (the layout of tj_fp64) <-> fused state.
template <typename R, int M>
__global__ void k_from_fp64(DevParams DP, MixB<R> b, const double* A, int* bad)
{
    const long long N = b.N;
    R* X = b.X[0];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int m = 0; m < M; ++m) {
            X[W_A(m) * N + g] = (R)A[(DP.S_ALPHA + m) * N + g];
            X[W_AR<M>(m) * N + g] = (R)A[(DP.S_ARHO + m) * N + g];
            X[W_RK<M>(m) * N + g] = (R)A[(DP.S_RHOK + m) * N + g];
        }
        for (int r = 0; r < 2; ++r) {
            X[W_RU<M>(r) * N + g] = (R)A[(DP.S_RHOU + r) * N + g];
            X[W_U<M>(r) * N + g] = (R)A[(DP.S_VEL + r) * N + g];
        }
        const double E = A[DP.S_E * N + g];
        const R eh = (R)E;
        X[W_EH<M>() * N + g] = eh;
        X[W_EL<M>() * N + g] = (R)(E - (double)eh);
        X[W_P<M>() * N + g] = (R)A[DP.S_P * N + g];
        if (A[(DP.S_VEL + 2) * N + g] != 0.0 || A[(DP.S_RHOU + 2) * N + g] != 0.0) atomicOr(bad, 1);
    }
}

// The whole domain in AccessPattern planes (component c of cell g at
// ap[c * N + g], with ngrow 0) -> the FP64 carried state and the fused state
// in one pass. ap may be a page-locked host buffer read in place: each thread
// issues all of a cell's loads before its stores, so that many are in flight
// over the host link. The values written are those of k_ap_to_state followed
// by k_from_fp64.
template <typename R, int M>
__global__ void k_from_ap(DevParams DP, MixB<R> b, const double* __restrict__ ap, double* __restrict__ A, int* bad)
{
    const long long N = b.N;
    R* __restrict__ X = b.X[0];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        double al[M], ar[M], rk[M], ru[3], u[3];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            al[m] = ap[(DP.A_ALPHA + m) * N + g];
            ar[m] = ap[(DP.A_ARHO + m) * N + g];
            rk[m] = ap[(DP.A_RHOK + m) * N + g];
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            ru[r] = ap[(DP.A_RHOU + r) * N + g];
            u[r] = ap[(DP.A_VEL + r) * N + g];
        }
        const double rho = ap[DP.A_RHO * N + g], E = ap[DP.A_E * N + g], p = ap[DP.A_P * N + g];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            A[(DP.S_ALPHA + m) * N + g] = al[m];
            A[(DP.S_ARHO + m) * N + g] = ar[m];
            A[(DP.S_RHOK + m) * N + g] = rk[m];
            X[W_A(m) * N + g] = (R)al[m];
            X[W_AR<M>(m) * N + g] = (R)ar[m];
            X[W_RK<M>(m) * N + g] = (R)rk[m];
        }
        A[DP.S_RHO * N + g] = rho;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            A[(DP.S_RHOU + r) * N + g] = ru[r];
            A[(DP.S_VEL + r) * N + g] = u[r];
        }
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            X[W_RU<M>(r) * N + g] = (R)ru[r];
            X[W_U<M>(r) * N + g] = (R)u[r];
        }
        A[DP.S_E * N + g] = E;
        const R eh = (R)E;
        X[W_EH<M>() * N + g] = eh;
        X[W_EL<M>() * N + g] = (R)(E - (double)eh);
        A[DP.S_P * N + g] = p;
        X[W_P<M>() * N + g] = (R)p;
        if (u[2] != 0.0 || ru[2] != 0.0) atomicOr(bad, 1);
    }
}

template <typename R, int M>
__global__ void k_to_fp64(DevParams DP, MixB<R> b, double* A)
{
    const long long N = b.N;
    const R* X = b.X[0];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        double rho = 0.0;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            A[(DP.S_ALPHA + m) * N + g] = X[W_A(m) * N + g];
            A[(DP.S_ARHO + m) * N + g] = X[W_AR<M>(m) * N + g];
            A[(DP.S_RHOK + m) * N + g] = X[W_RK<M>(m) * N + g];
            rho += (double)X[W_AR<M>(m) * N + g];
        }
        A[DP.S_RHO * N + g] = rho;
        for (int r = 0; r < 2; ++r) {
            A[(DP.S_RHOU + r) * N + g] = X[W_RU<M>(r) * N + g];
            A[(DP.S_VEL + r) * N + g] = X[W_U<M>(r) * N + g];
        }
        A[(DP.S_RHOU + 2) * N + g] = 0.0;
        A[(DP.S_VEL + 2) * N + g] = 0.0;
        A[DP.S_E * N + g] = (double)X[W_EH<M>() * N + g] + (double)X[W_EL<M>() * N + g];
        A[DP.S_P * N + g] = X[W_P<M>() * N + g];
    }
}

// End of a step (main.cpp:121 t += dt; NaN stop) and the THINC stage stamp.
__global__ void k_step_end_mixed(DevScalars* s, int* ctr)
{
    if (threadIdx.x != 0 || s->done) return;
    *ctr += 2;
    if (s->nan_flag) {
        s->done = 1;
        atomicCAS(&s->status, 0, TJ_ERR_NAN);
        return;
    }
    s->t += s->dt;
    s->n += 1;
}

__global__ void k_reset_dtmin(DevScalars* s)
{
    if (threadIdx.x == 0) s->dtmin_bits = 0x7FEFFFFFFFFFFFFFull;
}

static int nblk(long long n) { return (int)std::min<long long>((n + 255) / 256, 152 * 8); }

// ---------------------------------------------------------------------------
// Host side, per working type.
// ---------------------------------------------------------------------------
template <typename R>
struct MixedImpl : MixedBase {
    MixP<R> P;
    MixB<R> b;
    int M = 0, thinc = 0;
    R* X[2] = {nullptr, nullptr};
    R* starA[2] = {nullptr, nullptr};
    R* gstar[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    R* urv[2] = {nullptr, nullptr};
    int* urs[2] = {nullptr, nullptr};
    int* bx[4] = {nullptr, nullptr, nullptr, nullptr};
    int* ctr = nullptr;
    int* bad = nullptr;
    int* bad_h = nullptr;  // page-locked copy of bad

    ~MixedImpl() override
    {
        R* rs[] = {X[0], X[1], starA[0], starA[1], urv[0], urv[1], gstar[0][0], gstar[0][1], gstar[1][0], gstar[1][1]};
        for (R* p : rs)
            if (p) cudaFree(p);
        int* is[] = {urs[0], urs[1], bx[0], bx[1], bx[2], bx[3], ctr, bad};
        for (int* p : is)
            if (p) cudaFree(p);
        if (bad_h) cudaFreeHost(bad_h);
    }

    int alloc(const DevParams& DP, const DevDomain& D, long long N, cudaStream_t st)
    {
        M = DP.M;
        thinc = DP.thinc;
        std::memset(&P, 0, sizeof P);
        P.nx = D.n[0];
        P.ny = D.n[1];
        P.M = DP.M;
        P.thinc = DP.thinc;
        for (int d = 0; d < 2; ++d) {
            P.lo_bc[d] = DP.lo_bc[d];
            P.hi_bc[d] = DP.hi_bc[d];
            P.dx[d] = (R)D.dx[d];
            P.idx[d] = (R)(1.0 / D.dx[d]);
            P.dxd[d] = D.dx[d];
        }
        P.beta = (R)DP.beta;
        P.mxfloor = (R)1e-20;
        for (int k = 0; k < DP.M; ++k) {
            const double G = DP.prm[k][0] - 1.0;
            P.g[k] = (R)G;
            P.ig[k] = (R)(1.0 / G);
            P.pref[k] = (R)DP.prm[k][1];
            P.eref[k] = (R)DP.prm[k][2];
            const double cE = DP.prm[k][1] / G, eE = DP.prm[k][2];
            P.cEh[k] = (R)cE;
            P.cEl[k] = (R)(cE - (double)P.cEh[k]);
            P.eEh[k] = (R)eE;
            P.eEl[k] = (R)(eE - (double)P.eEh[k]);
        }
        const int NW = 3 * DP.M + 7;
        for (int q = 0; q < 2; ++q) {
            if (cudaMalloc(&X[q], sizeof(R) * NW * N) != cudaSuccess) return TJ_ERR_CUDA;
            cudaMemsetAsync(X[q], 0, sizeof(R) * NW * N, st);
        }
        if (DP.thinc) {
            const long long nf[2] = {(long long)(P.nx + 1) * P.ny, (long long)P.nx * (P.ny + 1)};
            for (int q = 0; q < 2; ++q) {
                if (cudaMalloc(&starA[q], sizeof(R) * DP.M * N) != cudaSuccess) return TJ_ERR_CUDA;
                cudaMemsetAsync(starA[q], 0, sizeof(R) * DP.M * N, st);
                if (cudaMalloc(&urv[q], sizeof(R) * DP.M * N) != cudaSuccess) return TJ_ERR_CUDA;
                cudaMemsetAsync(urv[q], 0, sizeof(R) * DP.M * N, st);
                if (cudaMalloc(&urs[q], sizeof(int) * DP.M * N) != cudaSuccess) return TJ_ERR_CUDA;
                cudaMemsetAsync(urs[q], 0xFF, sizeof(int) * DP.M * N, st);
                for (int d = 0; d < 2; ++d) {
                    if (cudaMalloc(&gstar[d][q], sizeof(R) * DP.M * nf[d]) != cudaSuccess) return TJ_ERR_CUDA;
                    cudaMemsetAsync(gstar[d][q], 0, sizeof(R) * DP.M * nf[d], st);
                }
            }
        }
        for (int d = 0; d < 2; ++d) {
            const int n = d == 0 ? P.nx : P.ny;
            if (cudaMalloc(&bx[2 * d], sizeof(int) * n) != cudaSuccess) return TJ_ERR_CUDA;
            if (cudaMalloc(&bx[2 * d + 1], sizeof(int) * n) != cudaSuccess) return TJ_ERR_CUDA;
        }
        if (cudaMalloc(&ctr, sizeof(int)) != cudaSuccess) return TJ_ERR_CUDA;
        cudaMemsetAsync(ctr, 0, sizeof(int), st);
        if (cudaMalloc(&bad, sizeof(int)) != cudaSuccess) return TJ_ERR_CUDA;
        cudaMemsetAsync(bad, 0, sizeof(int), st);
        if (cudaMallocHost(&bad_h, sizeof(int)) != cudaSuccess) return TJ_ERR_CUDA;
        *bad_h = 0;
        for (int q = 0; q < 2; ++q) {
            b.X[q] = X[q];
            b.starA[q] = starA[q];
            b.urv[q] = urv[q];
            b.urs[q] = urs[q];
            for (int d = 0; d < 2; ++d) b.gstar[d][q] = gstar[d][q];
        }
        b.bxlo[0] = bx[0];
        b.bxhi[0] = bx[1];
        b.bxlo[1] = bx[2];
        b.bxhi[1] = bx[3];
        b.stage_ctr = ctr;
        b.N = N;
        b.scal = nullptr;
        std::vector<int> one{0, 0, 0, P.nx - 1, P.ny - 1, 0};
        return set_boxes1(D, one, st);
    }

    int set_boxes(const std::vector<DevDomain>& doms, const std::vector<std::vector<int>>& boxes,
                  cudaStream_t st) override
    {
        return set_boxes1(doms[0], boxes[0], st);
    }

    int set_boxes1(const DevDomain& D, const std::vector<int>& bl, cudaStream_t st)
    {
        const int nb = (int)(bl.size() / 6);
        // the box list must be a tensor product of per-axis intervals
        std::vector<int> lo[2], hi[2];
        for (int d = 0; d < 2; ++d) {
            lo[d].assign(D.n[d], -1);
            hi[d].assign(D.n[d], -1);
        }
        for (int k = 0; k < nb; ++k) {
            const int* B = &bl[6 * k];
            for (int d = 0; d < 2; ++d)
                for (int i = B[d]; i <= B[3 + d]; ++i) {
                    if (lo[d][i] != -1 && (lo[d][i] != B[d] || hi[d][i] != B[3 + d])) return TJ_ERR_ARG;
                    lo[d][i] = B[d];
                    hi[d][i] = B[3 + d];
                }
        }
        for (int d = 0; d < 2; ++d) {
            cudaMemcpyAsync(bx[2 * d], lo[d].data(), sizeof(int) * D.n[d], cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(bx[2 * d + 1], hi[d].data(), sizeof(int) * D.n[d], cudaMemcpyHostToDevice, st);
        }
        const int* L = &bl[6 * (nb - 1)];
        P.last_box[0] = L[0];
        P.last_box[1] = L[1];
        P.last_box[2] = L[3];
        P.last_box[3] = L[4];
        cudaStreamSynchronize(st);
        return TJ_OK;
    }

    int from_fp64(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st) override
    {
        b.scal = fb.scal;
        cudaMemsetAsync(bad, 0, sizeof(int), st);
        switch (M) {
            case 1: k_from_fp64<R, 1><<<nblk(b.N), 256, 0, st>>>(DP, b, fb.A, bad); break;
            case 2: k_from_fp64<R, 2><<<nblk(b.N), 256, 0, st>>>(DP, b, fb.A, bad); break;
            case 3: k_from_fp64<R, 3><<<nblk(b.N), 256, 0, st>>>(DP, b, fb.A, bad); break;
            default: k_from_fp64<R, 4><<<nblk(b.N), 256, 0, st>>>(DP, b, fb.A, bad); break;
        }
        return 1 + cfl(fb, st) + report_w(st);
    }

    int from_ap(const DevParams& DP, const Fp64Bufs& fb, const double* ap, cudaStream_t st) override
    {
        b.scal = fb.scal;
        cudaMemsetAsync(bad, 0, sizeof(int), st);
        switch (M) {
            case 1: k_from_ap<R, 1><<<nblk(b.N), 256, 0, st>>>(DP, b, ap, fb.A, bad); break;
            case 2: k_from_ap<R, 2><<<nblk(b.N), 256, 0, st>>>(DP, b, ap, fb.A, bad); break;
            case 3: k_from_ap<R, 3><<<nblk(b.N), 256, 0, st>>>(DP, b, ap, fb.A, bad); break;
            default: k_from_ap<R, 4><<<nblk(b.N), 256, 0, st>>>(DP, b, ap, fb.A, bad); break;
        }
        return 1 + cfl(fb, st) + report_w(st);
    }

    // waits for the stream; warns when an uploaded cell had a third velocity
    // component, which the 2-D fused state does not carry
    int report_w(cudaStream_t st)
    {
        cudaMemcpyAsync(bad_h, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        if (*bad_h) std::fprintf(stderr, "tenjin_gpu: the fused 2-D kernels carry two velocity components; w was nonzero\n");
        return 0;
    }

    int to_fp64(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st) override
    {
        switch (M) {
            case 1: k_to_fp64<R, 1><<<nblk(b.N), 256, 0, st>>>(DP, b, fb.A); break;
            case 2: k_to_fp64<R, 2><<<nblk(b.N), 256, 0, st>>>(DP, b, fb.A); break;
            case 3: k_to_fp64<R, 3><<<nblk(b.N), 256, 0, st>>>(DP, b, fb.A); break;
            default: k_to_fp64<R, 4><<<nblk(b.N), 256, 0, st>>>(DP, b, fb.A); break;
        }
        return 1;
    }

    int cfl(const Fp64Bufs& fb, cudaStream_t st) override
    {
        b.scal = fb.scal;
        k_reset_dtmin<<<1, 32, 0, st>>>(fb.scal);
        switch (M) {
            case 1: k_cfl_mixed<R, 1><<<nblk(b.N), 256, 0, st>>>(P, b); break;
            case 2: k_cfl_mixed<R, 2><<<nblk(b.N), 256, 0, st>>>(P, b); break;
            case 3: k_cfl_mixed<R, 3><<<nblk(b.N), 256, 0, st>>>(P, b); break;
            default: k_cfl_mixed<R, 4><<<nblk(b.N), 256, 0, st>>>(P, b); break;
        }
        return 2;
    }

    template <int MM, bool TH>
    void launch_stage(int stage, cudaStream_t st)
    {
        static bool attr = false;
        const size_t smb = Smem<R, MM, TH>::BYTES;
        if (!attr) {
            cudaFuncSetAttribute(k_stage2d<R, MM, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb);
            attr = true;
        }
        dim3 grid((P.nx + MT - 1) / MT, (P.ny + MT - 1) / MT);
        k_stage2d<R, MM, TH><<<grid, NTH, smb, st>>>(P, b, stage);
    }

    void stage_dispatch(int stage, cudaStream_t st)
    {
        switch (M * 2 + (thinc ? 1 : 0)) {
            case 2: launch_stage<1, false>(stage, st); break;
            case 3: launch_stage<1, true>(stage, st); break;
            case 4: launch_stage<2, false>(stage, st); break;
            case 5: launch_stage<2, true>(stage, st); break;
            case 6: launch_stage<3, false>(stage, st); break;
            case 7: launch_stage<3, true>(stage, st); break;
            case 8: launch_stage<4, false>(stage, st); break;
            default: launch_stage<4, true>(stage, st); break;
        }
    }

    int step(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st, Prof* pr) override
    {
        b.scal = fb.scal;
        int n = 0;
        n += fp64_dt_finalize(DP, fb, 1, st);
        for (int stage = 0; stage < 2; ++stage) {
            if (pr) pr->begin(sizeof(R) == 4 ? "tj_stage_mixed" : "tj_stage_fused64", st);
            stage_dispatch(stage, st);
            if (pr) pr->end(sizeof(R) == 4 ? "tj_stage_mixed" : "tj_stage_fused64", st);
            n += 1;
        }
        k_step_end_mixed<<<1, 32, 0, st>>>(fb.scal, ctr);
        return n + 1;
    }
};

}  // namespace

// The fused 2-D kernels: one 2-D fluid domain with the stiffened-gas EOS.
static bool fused2d_covers(const DevParams& DP, size_t ndom)
{
    if (DP.dim != 2 || DP.solid || DP.plastic || DP.radial || ndom != 1 || DP.M > 4) return false;
    for (int m = 0; m < DP.M; ++m)
        if (DP.eos[m] != TJ_EOS_MIEGRUNEISEN || DP.phase[m] != TJ_PHASE_FLUID) return false;
    return true;
}

// The fused 3-D kernel: 3-D fluids with the stiffened-gas EOS, MUSCL (no THINC).
static bool fused3d_covers(const DevParams& DP)
{
    if (DP.dim != 3 || DP.solid || DP.plastic || DP.thinc || DP.radial || DP.M > 4) return false;
    for (int m = 0; m < DP.M; ++m)
        if (DP.eos[m] != TJ_EOS_MIEGRUNEISEN || DP.phase[m] != TJ_PHASE_FLUID) return false;
    return true;
}

bool mixed_supported(const tj_params& p)
{
    // binary32: every configuration (fused kernels where they apply, the
    // binary32 per-direction kernels otherwise); binary64 fused: 2-D fluids
    if (p.precision == TJ_PRECISION_MIXED) return true;
    if (p.dim != 2 || p.SOLID || p.PLASTIC || p.RADIAL) return false;
    if (p.n_materials < 1 || p.n_materials > 4) return false;
    for (int m = 0; m < p.n_materials; ++m)
        if (p.materials[m].eos != TJ_EOS_MIEGRUNEISEN || p.materials[m].phase != TJ_PHASE_FLUID) return false;
    return true;
}

int mixed_alloc(MixedState& ms, const DevParams& DP, const std::vector<DevDomain>& doms, long long ntot,
                const long long* nftot, cudaStream_t st)
{
    if (!DP.fused64 && fused3d_covers(DP)) {
        int err = TJ_OK;
        ms.impl = mixed3d_create(DP, doms, ntot, st, &err);
        ms.allocated = true;
        return err;
    }
    if (!DP.fused64 && !fused2d_covers(DP, doms.size())) {
        int err = TJ_OK;
        ms.impl = general32_create(DP, ntot, nftot, st, &err);
        ms.allocated = true;
        return err;
    }
    if (doms.size() != 1) return TJ_ERR_ARG;  // one 2-D domain
    if (DP.fused64) {
        auto* m = new MixedImpl<double>();
        ms.impl = m;
        ms.allocated = true;
        return m->alloc(DP, doms[0], ntot, st);
    }
    auto* m = new MixedImpl<float>();
    ms.impl = m;
    ms.allocated = true;
    return m->alloc(DP, doms[0], ntot, st);
}

void mixed_free(MixedState& ms)
{
    delete (MixedBase*)ms.impl;
    ms.impl = nullptr;
    ms.allocated = false;
}

int mixed_set_boxes(MixedState& ms, const DevParams& DP, const std::vector<DevDomain>& doms,
                    const std::vector<std::vector<int>>& boxes, cudaStream_t st)
{
    (void)DP;
    if (!ms.impl) return TJ_OK;
    return ((MixedBase*)ms.impl)->set_boxes(doms, boxes, st);
}

void mixed_describe(const MixedState& ms, char* buf, size_t len)
{
    if (!ms.impl) {
        if (len) buf[0] = 0;
        return;
    }
    ((const MixedBase*)ms.impl)->describe(buf, len);
}

int mixed_from_fp64(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st)
{
    return ((MixedBase*)ms.impl)->from_fp64(DP, fb, st);
}

int mixed_from_ap(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, const double* ap, cudaStream_t st)
{
    return ((MixedBase*)ms.impl)->from_ap(DP, fb, ap, st);
}

int mixed_to_fp64(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st)
{
    return ((MixedBase*)ms.impl)->to_fp64(DP, fb, st);
}

int mixed_compute_dt(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st)
{
    (void)DP;
    return ((MixedBase*)ms.impl)->cfl(fb, st);
}

int mixed_step(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st, Prof* pr)
{
    return ((MixedBase*)ms.impl)->step(DP, fb, st, pr);
}

int mixed_launches_per_step(const DevParams& DP)
{
    (void)DP;
    return 4;
}

}  // namespace tj
