// Mixed-precision fused stage kernel of the per-timestep update (2-D fluids).
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
// Arithmetic is binary32 except: the total energy is stored as a compensated
// pair of floats (hi + lo) and accumulated with an error-free sum; the
// pressure closure numerator E - KE - sum e_cold + sum p_cold, where the cold
// terms of a stiffened gas cancel E to four orders of magnitude, is evaluated
// in binary64 (boxaccesscellarray.cpp:116).
// BVD-THINC keeps the reference's scratch history: the alpha of the star
// state of the latest flux sweep (the reference's ULStar), the latest THINC
// right candidate of each cell (URStar, two stamped slots so that a stage
// never reads a value written in the same stage) and the star alpha at box
// hi+1 faces (ULStar's ghost), double-buffered by stage parity.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "tj_mixed.cuh"

namespace tj {

namespace {

constexpr int MT = 28;          // output tile edge
constexpr int MH = 3;           // staged halo
constexpr int MS = MT + 2 * MH;  // staged cells per axis (34)
constexpr int MP = MS + 1;       // shared-memory pitch (odd: conflict-free columns)
constexpr int CP = MT + 1;       // pitch of the output-cell arrays (odd)
constexpr int NTH = 256;         // threads per CTA
constexpr int NWARP = NTH / 32;
constexpr int XR0 = -2;          // first row (relative to y0) of the x sweep with THINC
constexpr int XRN = 32;          // rows of the x sweep with THINC: y0-2 .. y0+29

struct MixP {
    int nx, ny, M, thinc;
    int lo_bc[2], hi_bc[2];
    float dx[2], beta;
    float g[TJ_MAX_MAT], ig[TJ_MAX_MAT], pref[TJ_MAX_MAT], eref[TJ_MAX_MAT];
    // pref/Gamma and eref as float pairs (hi + lo) for the pressure closure
    float cEh[TJ_MAX_MAT], cEl[TJ_MAX_MAT], eEh[TJ_MAX_MAT], eEl[TJ_MAX_MAT];
    double cfl;
    int last_box[4];  // lo x, lo y, hi x, hi y of the last box in MFIter order
};

struct MixB {
    float* X[2];  // state buffers: 0 = U^n / result, 1 = stage-1 output
    float* starA[2];
    float* gstar[2][2];  // [direction][parity]
    float* urv[2];
    int* urs[2];
    const int* bxlo[2];
    const int* bxhi[2];
    DevScalars* scal;
    int* stage_ctr;
    long long N;
};

// word offsets of the mixed state
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

template <int M>
struct FaceS {
    float a[M], ar[M], rho, ru[2], u[2], E, p, c;
};

// MUSCL slope (hllc.cpp:527-568). With a = u0-um, b = up-u0 and r = a/b, the
// reference's limiter phi(r) = min(2/(1+r), 2r/(1+r)) for r > 0 (0 for r <= 0,
// inf or NaN) applied to (up-um)/2 equals, in exact arithmetic, the argument
// of smaller magnitude when a and b have the same sign and 0 otherwise; the
// binary32 path evaluates that division-free form.
__device__ __forceinline__ void muscl_f(float um, float u0, float up, float& l, float& r)
{
    const float a = u0 - um, b = up - u0;
    float g = 0.f;
    if (a * b > 0.f) g = (fabsf(a) < fabsf(b)) ? a : b;
    l = u0 - 0.5f * g;
    r = u0 + 0.5f * g;
}

// Error-free product of a float by a float pair (ch + cl): returns hi, adds
// the rounding error and the low-part product to lo.
__device__ __forceinline__ float two_prod_acc(float ch, float cl, float x, float& lo)
{
    const float p = ch * x;
    lo += fmaf(ch, x, -p) + cl * x;
    return p;
}

// Error-free sum of two floats: s + e == a + b exactly.
__device__ __forceinline__ float two_sum(float a, float b, float& e)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

// Error-free accumulation of a float into a (hi, lo) pair.
__device__ __forceinline__ void dd_add(float& hi, float& lo, float b)
{
    float s = __fadd_rn(hi, b);
    float bb = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    lo = __fadd_rn(lo, e);
    float t = __fadd_rn(s, lo);
    lo = __fsub_rn(lo, __fsub_rn(t, s));
    hi = t;
}

template <int M>
__device__ __forceinline__ void cleanup_f(float* a)
{
    float tot = 0.f;
    int nan = 0;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        float v = a[m];
        if (isnan(v)) {
            v = 0.f;
            if (nan == 0) nan = m;
        } else if (v < 0.f) v = 1e-6f;
        else if (v > 1.f) v = 1.f;
        a[m] = v;
        tot += v;
    }
    if (nan > 0) {
        a[nan] = 1.f - tot;
        tot += a[nan];
    }
    float it = 1.f / tot;
#pragma unroll
    for (int m = 0; m < M; ++m) a[m] *= it;
}

// primitiveToConservative + getSoundSpeed of a reconstructed state.
template <int M>
__device__ __forceinline__ void p2c_f(const MixP& P, const float* rk, FaceS<M>& s)
{
    s.rho = 0.f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        s.ar[m] = s.a[m] * rk[m];
        s.rho += s.ar[m];
    }
    float ke = 0.f;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        s.ru[r] = s.u[r] * s.rho;
        ke += 0.5f * s.rho * s.u[r] * s.u[r];
    }
    float G = 0.f, ec = 0.f, pc = 0.f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        G += s.a[m] * P.ig[m];
        ec += P.eref[m] * s.ar[m];
        pc += P.pref[m] * s.a[m] * P.ig[m];
    }
    s.E = s.p * G + ec - pc + ke;
    float sa = 0.f, xt = 0.f;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        float c2 = s.p * (P.g[m] + 1.f) / rk[m] - P.pref[m] / rk[m];
        float v = P.ig[m] * c2 * s.ar[m] / s.rho;
        sa += (0.f < v) ? v : 0.f;
        xt += P.ig[m] * s.a[m];
    }
    if (sa <= 0.f) sa = 1e-6f;
    s.c = sqrtf(sa / xt);
}

template <int M>
struct Flux {
    float f[2 * M + 4];  // alpha[M], alphaRho[M], rhoU (2), E; f[2M+3] = S*
};

// HLLC flux of one face (hllc.cpp:384-487); returns the side whose star
// alpha the face carries (0 left, 1 right).
template <int M>
__device__ __forceinline__ int hllc_f(const FaceS<M>& L, const FaceS<M>& R, int d, Flux<M>& F)
{
    float x1 = fabsf(L.u[d]) + L.c, x2 = fabsf(R.u[d]) + R.c;
    float SR = (x1 < x2) ? x2 : x1;
    float SL = -SR;
    float Ss = (R.p - L.p + L.ru[d] * (SL - L.u[d]) - R.ru[d] * (SR - R.u[d])) /
               (L.rho * (SL - L.u[d]) - R.rho * (SR - R.u[d]));
    F.f[2 * M + 3] = Ss;
    const bool left = (SL >= 0.f) || (Ss >= 0.f);
    const bool hllc = left ? !(SL >= 0.f) : (SR >= 0.f);
    const FaceS<M>& K = left ? L : R;
    const float SK = left ? SL : SR;
    const float uK = K.u[d];
    float mult = (fabsf((Ss - uK) / Ss) < 1e-20f) ? 1.f : (SK - uK) / (SK - Ss);
    float rs = 0.f, ars[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        ars[m] = mult * K.ar[m];
        rs += ars[m];
    }
    float rus[2];
    rus[d] = mult * K.rho * Ss;
    rus[1 - d] = mult * K.ru[1 - d];
    float usd = rus[d] / rs;
    float Es = mult * K.rho * (K.E / K.rho + (Ss - uK) * (Ss + K.p / (K.rho * (SK - uK))));
    float w = hllc ? SK : 0.f;
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

struct Cand {
    unsigned mask;
    float L[TJ_MAX_MAT], R[TJ_MAX_MAT];
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

__device__ __forceinline__ float ur_read(const MixB& b, int m, long long c, int s)
{
    const long long k = (long long)m * b.N + c;
    int s0 = b.urs[0][k], s1 = b.urs[1][k];
    float v = 0.f;
    int best = -1;
    if (s0 < s && s0 > best) { best = s0; v = b.urv[0][k]; }
    if (s1 < s && s1 > best) { v = b.urv[1][k]; }
    return v;
}

__device__ __forceinline__ void ur_write(const MixB& b, int m, long long c, int s, float v)
{
    const long long k = (long long)m * b.N + c;
    int slot = (b.urs[0][k] <= b.urs[1][k]) ? 0 : 1;
    b.urv[slot][k] = v;
    b.urs[slot][k] = s;
}

// Shared-memory layout of one CTA.
template <int M, bool THINC>
struct Smem {
    static constexpr int NP = NPRIM<M>();
    static constexpr int NC = 2 * M + 4;  // alpha[M], alphaRho[M], rhoU(2), E hi, E lo
    static constexpr int U_OFF = 0;
    static constexpr int CT = MT * CP;    // one output-cell plane
    static constexpr int C_OFF = U_OFF + NP * MS * MP;
    static constexpr int SAX_OFF = C_OFF + NC * CT;                        // star alpha of x faces, rows y0-1..y0+29
    static constexpr int CRX_OFF = SAX_OFF + (THINC ? M * 31 * CP : 0);    // x right candidates, rows y0-2..y0+28
    static constexpr int MX_OFF = CRX_OFF + (THINC ? M * 31 * CP : 0);     // x mixed masks (as float bits)
    static constexpr int SAY_OFF = MX_OFF + (THINC ? 31 * CP : 0);         // star alpha of y faces (output cells)
    static constexpr int URV_OFF = SAY_OFF + (THINC ? M * CT : 0);         // new URStar values
    static constexpr int URF_OFF = URV_OFF + (THINC ? M * CT : 0);         // new URStar mask
    static constexpr int RED_OFF = URF_OFF + (THINC ? CT : 0);
    static constexpr int TOTAL = RED_OFF + 32;
    static constexpr size_t BYTES = sizeof(float) * TOTAL;
};

// The THINC candidate of the cell at staged position (tx, ty) along d.
template <int M>
__device__ __forceinline__ void thinc_cand_f(const MixP& P, const float* sU, int tx, int ty, int d, Cand& c)
{
    const int ox = d == 0 ? 1 : 0, oy = d == 0 ? 0 : 1;
    c.mask = 0;
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const float* A = sU + m * MS * MP;
        float aL = A[(ty - oy) * MP + tx - ox], aR = A[(ty + oy) * MP + tx + ox], a0 = A[ty * MP + tx];
        float mn = (aR < aL) ? aR : aL;
        float mx = ((aL < aR) ? aR : aL) - mn;
        float theta = (float)((0.f < aR - aL) - (aR - aL < 0.f));
        // C = (a0-mn+eps)/(mx+eps) (0 when mx < eps); the interval test is
        // made on the numerator so that the division is only done when mixed
        const float num = a0 - mn + 1e-20f, den = mx + 1e-20f;
        bool mixed = !(mx < 1e-20f) && (num > 1e-4f * den) && (num < (0.999999f - 1e-4f) * den) &&
                     ((aR - a0) * (a0 - aL) >= 0.f);
        c.L[m] = 0.f;
        c.R[m] = 0.f;
        if (mixed) {
            const float C = num / den;
            c.mask |= 1u << m;
            float nx = -1.f / (8.f * P.dx[0]) *
                       (A[(ty + 1) * MP + tx + 1] + 2.f * A[ty * MP + tx + 1] + A[(ty - 1) * MP + tx + 1] -
                        A[(ty + 1) * MP + tx - 1] - 2.f * A[ty * MP + tx - 1] - A[(ty - 1) * MP + tx - 1]);
            float ny = -1.f / (8.f * P.dx[1]) *
                       (A[(ty + 1) * MP + tx + 1] + 2.f * A[(ty + 1) * MP + tx] + A[(ty + 1) * MP + tx - 1] -
                        A[(ty - 1) * MP + tx - 1] - 2.f * A[(ty - 1) * MP + tx] - A[(ty - 1) * MP + tx + 1]);
            float norm = sqrtf(nx * nx + ny * ny);
            float nvc = (norm < 1e-20f) ? 0.f : fabsf((d == 0 ? nx : ny) / norm);
            float beta = nvc * P.beta + 0.01f;
            float coshB = coshf(beta), tanhB = tanhf(beta);
            float B = expf(theta * beta * ((2.f * C) - 1.f));
            float Aa = ((B / coshB) - 1.f) / tanhB;
            c.R[m] = mn + (mx / 2.f) * (1.f + theta * ((tanhB + Aa) / (1.f + Aa * tanhB)));
            c.L[m] = mn + (mx / 2.f) * (1.f + theta * Aa);
        }
    }
}

// One sweep line (a row for d = 0, a column for d = 1) of 32 lanes.
// line: y (d=0) or x (d=1) of the line; p0: first lane position along d.
template <int M, bool THINC, int D>
__device__ void sweep_line(const MixP& P, const MixB& b, float* sm, int x0, int y0, int line, int s, float dtdx,
                           bool want_flux)
{
    using SM = Smem<M, THINC>;
    const float* sU = sm + SM::U_OFF;
    const int lane = threadIdx.x & 31;
    const int n = D == 0 ? P.nx : P.ny;
    const int p0 = (D == 0 ? x0 : y0) - 2;
    const int pos = p0 + lane;  // cell position along d
    // staged coordinates of this lane's cell
    const int tx = D == 0 ? lane + 1 : line - x0 + MH;
    const int ty = D == 0 ? line - y0 + MH : lane + 1;
    const int ox = D == 0 ? 1 : 0, oy = D == 0 ? 0 : 1;
    constexpr int NP = NPRIM<M>();
    float ul[NP], ur[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
        const float* Q = sU + q * MS * MP;
        float um = Q[(ty - oy) * MP + tx - ox], u0 = Q[ty * MP + tx], up = Q[(ty + oy) * MP + tx + ox];
        muscl_f(um, u0, up, ul[q], ur[q]);
    }
    // ---- BVD-THINC (thinc.cpp:67-208) ----
    Cand cd;
    cd.mask = 0;
    const bool valid = pos >= 0 && pos < n;
    if (THINC) thinc_cand_f<M>(P, sU, tx, ty, D, cd);
    const bool flag = THINC && ((cd.mask >> (M - 1)) & 1u);
    // the TBV comparison only runs in lines that hold a flagged cell
    if (THINC && __any_sync(0xffffffffu, flag && valid && lane >= 1 && lane <= 30)) {
        unsigned mm = __shfl_up_sync(0xffffffffu, cd.mask, 1), mp = __shfl_down_sync(0xffffffffu, cd.mask, 1);
        const int lo = valid ? b.bxlo[D][pos] : 0, hi = valid ? b.bxhi[D][pos] : -1;
        const bool in_m = valid && pos - 1 >= lo, in_p = valid && pos + 1 <= hi;
        const int cx = D == 0 ? pos : line, cy = D == 0 ? line : pos;
        const long long cell = cx + (long long)P.nx * cy;
        const int par_in = (s + 1) & 1;
        bool need = flag && valid && lane >= 1 && lane <= 30;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            float urm_m = __shfl_up_sync(0xffffffffu, ur[m], 1);     // MUSCL UR alpha of pos-1
            float ulp_m = __shfl_down_sync(0xffffffffu, ul[m], 1);   // MUSCL UL alpha of pos+1
            float cRm = __shfl_up_sync(0xffffffffu, cd.R[m], 1);
            float cLp = __shfl_down_sync(0xffffffffu, cd.L[m], 1);
            if (!need) continue;
            const float* A = sU + m * MS * MP;
            float urm, ulp, trm, tlp;
            if (in_m) {
                urm = urm_m;
                if ((mm >> m) & 1u) trm = cRm;
                else {
                    // URStar before this sweep at pos-1
                    if (D == 0) trm = ur_read(b, m, cell - 1, s);
                    else {
                        const int r = pos - 1 - (y0 - 2);
                        const float* CRX = sm + SM::CRX_OFF;
                        const unsigned mx = __float_as_uint(sm[SM::MX_OFF + r * CP + (line - x0)]);
                        trm = ((mx >> m) & 1u) ? CRX[(m * 31 + r) * CP + (line - x0)] : ur_read(b, m, cell - P.nx, s);
                    }
                }
            } else {
                urm = A[(ty - oy) * MP + tx - ox];
                trm = 0.f;
            }
            if (in_p) {
                ulp = ulp_m;
                if ((mp >> m) & 1u) tlp = cLp;
                else if (D == 0) tlp = b.starA[par_in][(long long)m * b.N + cell + 1];
                else tlp = sm[SM::SAX_OFF + (m * 31 + (pos + 1 - (y0 - 1))) * CP + (line - x0)];
            } else {
                ulp = A[(ty + oy) * MP + tx + ox];
                const long long f = D == 0 ? (pos + 1) + (long long)(P.nx + 1) * line : line + (long long)P.nx * (pos + 1);
                tlp = b.gstar[D][par_in][(long long)m * (D == 0 ? (long long)(P.nx + 1) * P.ny : (long long)P.nx * (P.ny + 1)) + f];
            }
            float tpl, tpr;
            if ((cd.mask >> m) & 1u) {
                tpl = cd.L[m];
                tpr = cd.R[m];
            } else if (D == 0) {
                tpl = b.starA[par_in][(long long)m * b.N + cell];
                tpr = ur_read(b, m, cell, s);
            } else {
                const int r = pos - (y0 - 2);
                const unsigned mx = __float_as_uint(sm[SM::MX_OFF + r * CP + (line - x0)]);
                tpl = sm[SM::SAX_OFF + (m * 31 + (pos - (y0 - 1))) * CP + (line - x0)];
                tpr = ((mx >> m) & 1u) ? sm[SM::CRX_OFF + (m * 31 + r) * CP + (line - x0)] : ur_read(b, m, cell, s);
            }
            float upl = ul[m], upr = ur[m];
#define MNF(a_, b_) (((b_) < (a_)) ? (b_) : (a_))
#define TBVF(PL, PR)                                                                          \
    MNF(MNF(fabsf(urm - (PL)) + fabsf((PR)-ulp), fabsf(trm - (PL)) + fabsf((PR)-tlp)),        \
        MNF(fabsf(urm - (PL)) + fabsf((PR)-tlp), fabsf(trm - (PL)) + fabsf((PR)-ulp)))
            float tm_ = TBVF(upl, upr), tt_ = TBVF(tpl, tpr);
#undef TBVF
#undef MNF
            if (tt_ < tm_) {
                ul[m] = tpl;
                ur[m] = tpr;
            }
        }
    }
    // ---- cleanUpAlpha, primitiveToConservative, getSoundSpeed ----
    FaceS<M> SLs, SRs;
    float rkl[M], rkr[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        SLs.a[m] = ul[m];
        SRs.a[m] = ur[m];
        rkl[m] = ul[M + m];
        rkr[m] = ur[M + m];
    }
    if (THINC) {
        cleanup_f<M>(SLs.a);
        cleanup_f<M>(SRs.a);
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        SLs.u[r] = ul[2 * M + r];
        SRs.u[r] = ur[2 * M + r];
    }
    SLs.p = ul[2 * M + 2];
    SRs.p = ur[2 * M + 2];
    p2c_f<M>(P, rkl, SLs);
    p2c_f<M>(P, rkr, SRs);

    // ---- ghost lanes take the boundary image of a valid lane's state ----
    bool refl;
    const int lo_bc = P.lo_bc[D], hi_bc = P.hi_bc[D];
    const int src = reflect_map(pos, n, lo_bc, hi_bc, refl);
    const int src_lane = src - p0;
    if (p0 < 0 || p0 + 31 >= n) {  // only lines that reach the domain boundary
        const int sl = (src_lane >= 0 && src_lane < 32) ? src_lane : lane;
        FaceS<M>* S2[2] = {&SLs, &SRs};
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            FaceS<M>& S = *S2[side];
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
            sm[SM::MX_OFF + r * CP + (pos - x0)] = __uint_as_float(cd.mask);
#pragma unroll
            for (int m = 0; m < M; ++m) sm[SM::CRX_OFF + (m * 31 + r) * CP + (pos - x0)] = cd.R[m];
        }
    }
    if (!want_flux) return;

    // ---- flux of the lower face: left state UR of pos-1, right state UL of pos ----
    FaceS<M> Lf;
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
    Flux<M> F;
    int side = hllc_f<M>(Lf, SLs, D, F);
    float astar[M];
#pragma unroll
    for (int m = 0; m < M; ++m) astar[m] = side ? SLs.a[m] : Lf.a[m];

    // the face is owned by this tile if its right cell is an output cell, or
    // if it is the domain's hi face and its left cell is an output cell
    const bool hi_face = pos == n && lane >= 3 && lane <= 30;
    if (THINC) {
        // star alpha: x faces kept in shared memory (rows y0-1..y0+29) for
        // the y sweep; y faces of output cells go out as the next stage's ULStar
        if (D == 0) {
            const int r = line - (y0 - 1);
            if (r >= 0 && r < 31 && out_cell)
#pragma unroll
                for (int m = 0; m < M; ++m) sm[SM::SAX_OFF + (m * 31 + r) * CP + (pos - x0)] = astar[m];
        } else if (out_cell) {
#pragma unroll
            for (int m = 0; m < M; ++m) sm[SM::SAY_OFF + m * SM::CT + (pos - y0) * CP + (line - x0)] = astar[m];
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
            const int r = pos - (y0 - 2);
            const unsigned mxm = __float_as_uint(sm[SM::MX_OFF + r * CP + (line - x0)]);
            unsigned f = cd.mask | mxm;
#pragma unroll
            for (int m = 0; m < M; ++m) {
                float v = ((cd.mask >> m) & 1u) ? cd.R[m] : sm[SM::CRX_OFF + (m * 31 + r) * CP + (line - x0)];
                sm[SM::URV_OFF + m * SM::CT + (pos - y0) * CP + (line - x0)] = v;
            }
            sm[SM::URF_OFF + (pos - y0) * CP + (line - x0)] = __uint_as_float(f);
        }
    }

    // ---- update of the lane's cell: needs the flux of the upper face ----
    float fu[2 * M + 4];
#pragma unroll
    for (int q = 0; q < 2 * M + 4; ++q) fu[q] = __shfl_down_sync(0xffffffffu, F.f[q], 1);
    const bool upd_line = D == 0 ? (line >= y0 && line < y0 + MT && line < P.ny) : true;
    if (!(out_cell && upd_line)) return;
    const int ci = D == 0 ? pos - x0 : line - x0;  // output tile column
    const int cj = D == 0 ? line - y0 : pos - y0;  // output tile row
    float* C = sm + SM::C_OFF;
    const int oc = cj * CP + ci;
    constexpr int MTT = MT * CP;
    const float dS = F.f[2 * M + 3] - fu[2 * M + 3];
#pragma unroll
    for (int m = 0; m < M; ++m) {
        const float a0 = sU[m * MS * MP + ty * MP + tx];
        C[m * MTT + oc] += dtdx * (F.f[m] - fu[m] - a0 * dS);
        C[(M + m) * MTT + oc] += dtdx * (F.f[M + m] - fu[M + m]);
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) C[(2 * M + r) * MTT + oc] += dtdx * (F.f[2 * M + r] - fu[2 * M + r]);
    float eh = C[(2 * M + 2) * MTT + oc], el = C[(2 * M + 3) * MTT + oc];
    dd_add(eh, el, dtdx * (F.f[2 * M + 2] - fu[2 * M + 2]));
    C[(2 * M + 2) * MTT + oc] = eh;
    C[(2 * M + 3) * MTT + oc] = el;
}

template <int M, bool THINC>
__global__ void __launch_bounds__(NTH, 2) k_stage2d(MixP P, MixB b, int stage)
{
    if (b.scal->done) return;
    using SM = Smem<M, THINC>;
    extern __shared__ float sm[];
    constexpr int NP = NPRIM<M>();
    constexpr int NW = NWORDS<M>();
    const int x0 = blockIdx.x * MT, y0 = blockIdx.y * MT;
    const int s = *b.stage_ctr;
    const float* __restrict__ Xin = b.X[stage];
    float* __restrict__ Xout = b.X[stage == 0 ? 1 : 0];
    const long long N = b.N;
    const float dtdx = (float)(b.scal->dt / (double)P.dx[0]);
    const float dtdy = (float)(b.scal->dt / (double)P.dx[1]);

    // ---- stage the primitives of tile + halo ----
    for (int t = threadIdx.x; t < MS * MS; t += NTH) {
        const int tx = t % MS, ty = t / MS;
        bool rx, ry;
        const int gx = reflect_map(x0 - MH + tx, P.nx, P.lo_bc[0], P.hi_bc[0], rx);
        const int gy = reflect_map(y0 - MH + ty, P.ny, P.lo_bc[1], P.hi_bc[1], ry);
        const long long g = gx + (long long)P.nx * gy;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            sm[SM::U_OFF + m * MS * MP + ty * MP + tx] = Xin[W_A(m) * N + g];
            sm[SM::U_OFF + (M + m) * MS * MP + ty * MP + tx] = Xin[W_RK<M>(m) * N + g];
        }
        float u = Xin[W_U<M>(0) * N + g], v = Xin[W_U<M>(1) * N + g];
        sm[SM::U_OFF + (2 * M) * MS * MP + ty * MP + tx] = rx ? -u : u;
        sm[SM::U_OFF + (2 * M + 1) * MS * MP + ty * MP + tx] = ry ? -v : v;
        sm[SM::U_OFF + (2 * M + 2) * MS * MP + ty * MP + tx] = Xin[W_P<M>() * N + g];
    }
    // ---- conserved variables of the output cells: U1 = U (hllc.cpp:583) ----
    for (int t = threadIdx.x; t < MT * MT; t += NTH) {
        const int ci = t % MT, cj = t / MT;
        const int gx = x0 + ci, gy = y0 + cj;
        if (gx >= P.nx || gy >= P.ny) continue;
        const long long g = gx + (long long)P.nx * gy;
        const int oc = cj * CP + ci;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            sm[SM::C_OFF + m * SM::CT + oc] = Xin[W_A(m) * N + g];
            sm[SM::C_OFF + (M + m) * SM::CT + oc] = Xin[W_AR<M>(m) * N + g];
        }
        sm[SM::C_OFF + (2 * M) * SM::CT + oc] = Xin[W_RU<M>(0) * N + g];
        sm[SM::C_OFF + (2 * M + 1) * SM::CT + oc] = Xin[W_RU<M>(1) * N + g];
        sm[SM::C_OFF + (2 * M + 2) * SM::CT + oc] = Xin[W_EH<M>() * N + g];
        sm[SM::C_OFF + (2 * M + 3) * SM::CT + oc] = Xin[W_EL<M>() * N + g];
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5;
    // ---- x sweep: rows ----
    {
        const int r0 = THINC ? y0 + XR0 : y0;
        const int nr = THINC ? XRN : MT;
        for (int r = warp; r < nr; r += NWARP) {
            const int line = r0 + r;
            if (line < 0 || line >= P.ny) continue;
            sweep_line<M, THINC, 0>(P, b, sm, x0, y0, line, s, dtdx, !THINC || line >= y0 - 1);
        }
    }
    __syncthreads();
    // ---- y sweep: columns ----
    for (int c = warp; c < MT; c += NWARP) {
        const int line = x0 + c;
        if (line >= P.nx) continue;
        sweep_line<M, THINC, 1>(P, b, sm, x0, y0, line, s, dtdy, true);
    }
    __syncthreads();

    // ---- finish: c2p; stage 2: average, cleanUpAlpha, CFL, NaN check ----
    float dtmin = 3.0e38f;
    bool nan_seen = false;
    for (int t = threadIdx.x; t < MT * MT; t += NTH) {
        const int ci = t % MT, cj = t / MT;
        const int gx = x0 + ci, gy = y0 + cj;
        if (gx >= P.nx || gy >= P.ny) continue;
        const long long g = gx + (long long)P.nx * gy;
        const int oc = cj * CP + ci;
        float a[M], ar[M], rk[M], ru[2], u[2], eh, el, p;
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
        float rho = 0.f;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            rk[m] = ar[m] / a[m];
            rho += ar[m];
        }
        float ke = 0.f;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            u[r] = ru[r] / rho;
            ke += 0.5f * rho * u[r] * u[r];
        }
        // p = (E - KE - sum e_cold + sum p_cold) / sum alpha/Gamma
        // (boxaccesscellarray.cpp:116). The cold terms of a stiffened gas
        // cancel E to four orders of magnitude, so the numerator is carried
        // as an unevaluated float pair (error-free sums and products).
        float sh = eh, sl = el, e, lo;
        sh = two_sum(sh, -ke, e);
        sl += e;
        float G = 0.f;
#pragma unroll
        for (int m = 0; m < M; ++m) {
            lo = 0.f;
            const float ec = two_prod_acc(P.eEh[m], P.eEl[m], ar[m], lo);
            sh = two_sum(sh, -ec, e);
            sl += e - lo;
            lo = 0.f;
            const float pc = two_prod_acc(P.cEh[m], P.cEl[m], a[m], lo);
            sh = two_sum(sh, pc, e);
            sl += e + lo;
            G += a[m] * P.ig[m];
        }
        p = (sh + sl) / G;
        if (stage == 1) {
            // U1 = U*0.5 + U2*0.5 over the carried state (hllc.cpp:705)
#pragma unroll
            for (int m = 0; m < M; ++m) {
                a[m] = 0.5f * Xout[W_A(m) * N + g] + 0.5f * a[m];
                ar[m] = 0.5f * Xout[W_AR<M>(m) * N + g] + 0.5f * ar[m];
                rk[m] = 0.5f * Xout[W_RK<M>(m) * N + g] + 0.5f * rk[m];
            }
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                ru[r] = 0.5f * Xout[W_RU<M>(r) * N + g] + 0.5f * ru[r];
                u[r] = 0.5f * Xout[W_U<M>(r) * N + g] + 0.5f * u[r];
            }
            p = 0.5f * Xout[W_P<M>() * N + g] + 0.5f * p;
            float h0 = Xout[W_EH<M>() * N + g], l0 = Xout[W_EL<M>() * N + g];
            float hs = 0.5f * h0, ls = 0.5f * l0;
            dd_add(hs, ls, 0.5f * eh);
            ls += 0.5f * el;
            float tt = hs + ls;
            el = ls - (tt - hs);
            eh = tt;
            cleanup_f<M>(a);  // main.cpp:170
            // next step's CFL (timestep.cpp:7-29), rho = sum alphaRho
            float rr = 0.f, sa = 0.f, xt = 0.f;
#pragma unroll
            for (int m = 0; m < M; ++m) rr += ar[m];
#pragma unroll
            for (int m = 0; m < M; ++m) {
                float c2 = p * (P.g[m] + 1.f) / rk[m] - P.pref[m] / rk[m];
                float v = P.ig[m] * c2 * ar[m] / rr;
                sa += (0.f < v) ? v : 0.f;
                xt += P.ig[m] * a[m];
            }
            if (sa <= 0.f) sa = 1e-6f;
            float cs = sqrtf(sa / xt);
            float v0 = P.dx[0] / (cs + fabsf(u[0])), v1 = P.dx[1] / (cs + fabsf(u[1]));
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
        if (THINC) {
            const int par_out = s & 1;
#pragma unroll
            for (int m = 0; m < M; ++m) b.starA[par_out][(long long)m * N + g] = sm[SM::SAY_OFF + m * SM::CT + oc];
            const unsigned f = __float_as_uint(sm[SM::URF_OFF + oc]);
            if (f)
#pragma unroll
                for (int m = 0; m < M; ++m)
                    if ((f >> m) & 1u) ur_write(b, m, g, s, sm[SM::URV_OFF + m * SM::CT + oc]);
        }
    }
    (void)NP;
    (void)NW;
    if (stage == 1) {
        if (nan_seen) atomicOr(&b.scal->nan_flag, 1);
        for (int o = 16; o > 0; o >>= 1) {
            float w = __shfl_down_sync(0xffffffffu, dtmin, o);
            dtmin = (w < dtmin) ? w : dtmin;
        }
        float* red = sm + SM::RED_OFF;
        const int lane = threadIdx.x & 31;
        __syncthreads();
        if (lane == 0) red[warp] = dtmin;
        __syncthreads();
        if (threadIdx.x == 0) {
            float mn = red[0];
            for (int w = 1; w < NWARP; ++w) mn = (red[w] < mn) ? red[w] : mn;
            atomicMin(&b.scal->dtmin_bits, (unsigned long long)__double_as_longlong((double)mn));
        }
    }
}

// CFL of the current mixed state (used after the state is set from outside).
template <int M>
__global__ void k_cfl_mixed(MixP P, MixB b)
{
    float dtmin = 3.0e38f;
    const long long N = b.N;
    const float* X = b.X[0];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
        float rr = 0.f, sa = 0.f, xt = 0.f, ar[M], a[M], rk[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            a[m] = X[W_A(m) * N + g];
            ar[m] = X[W_AR<M>(m) * N + g];
            rk[m] = X[W_RK<M>(m) * N + g];
            rr += ar[m];
        }
        const float p = X[W_P<M>() * N + g];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            float c2 = p * (P.g[m] + 1.f) / rk[m] - P.pref[m] / rk[m];
            float v = P.ig[m] * c2 * ar[m] / rr;
            sa += (0.f < v) ? v : 0.f;
            xt += P.ig[m] * a[m];
        }
        if (sa <= 0.f) sa = 1e-6f;
        float cs = sqrtf(sa / xt);
        float v0 = P.dx[0] / (cs + fabsf(X[W_U<M>(0) * N + g])), v1 = P.dx[1] / (cs + fabsf(X[W_U<M>(1) * N + g]));
        dtmin = fminf(dtmin, fminf(v0, v1));
    }
    for (int o = 16; o > 0; o >>= 1) dtmin = fminf(dtmin, __shfl_down_sync(0xffffffffu, dtmin, o));
    if ((threadIdx.x & 31) == 0) atomicMin(&b.scal->dtmin_bits, (unsigned long long)__double_as_longlong((double)dtmin));
}

// FP64 carried state (the reference layout of tj_fp64) <-> mixed state.
template <int M>
__global__ void k_from_fp64(DevParams DP, MixB b, const double* A, int* bad)
{
    const long long N = b.N;
    float* X = b.X[0];
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N; g += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int m = 0; m < M; ++m) {
            X[W_A(m) * N + g] = (float)A[(DP.S_ALPHA + m) * N + g];
            X[W_AR<M>(m) * N + g] = (float)A[(DP.S_ARHO + m) * N + g];
            X[W_RK<M>(m) * N + g] = (float)A[(DP.S_RHOK + m) * N + g];
        }
        for (int r = 0; r < 2; ++r) {
            X[W_RU<M>(r) * N + g] = (float)A[(DP.S_RHOU + r) * N + g];
            X[W_U<M>(r) * N + g] = (float)A[(DP.S_VEL + r) * N + g];
        }
        const double E = A[DP.S_E * N + g];
        const float eh = (float)E;
        X[W_EH<M>() * N + g] = eh;
        X[W_EL<M>() * N + g] = (float)(E - (double)eh);
        X[W_P<M>() * N + g] = (float)A[DP.S_P * N + g];
        if (A[(DP.S_VEL + 2) * N + g] != 0.0 || A[(DP.S_RHOU + 2) * N + g] != 0.0) atomicOr(bad, 1);
    }
}

template <int M>
__global__ void k_to_fp64(DevParams DP, MixB b, double* A)
{
    const long long N = b.N;
    const float* X = b.X[0];
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

__global__ void k_stage_ctr_inc(int* ctr, DevScalars* s)
{
    if (threadIdx.x == 0 && !s->done) *ctr += 1;
}

__global__ void k_reset_dtmin(DevScalars* s)
{
    if (threadIdx.x == 0) s->dtmin_bits = 0x7FEFFFFFFFFFFFFFull;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct MixedImpl {
    MixP P;
    MixB b;
    int M = 0, thinc = 0;
    float* X[2] = {nullptr, nullptr};
    float* starA[2] = {nullptr, nullptr};
    float* gstar[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    float* urv[2] = {nullptr, nullptr};
    int* urs[2] = {nullptr, nullptr};
    int* bx[4] = {nullptr, nullptr, nullptr, nullptr};
    int* ctr = nullptr;
    int* bad = nullptr;
};

bool mixed_supported(const tj_params& p)
{
    if (p.dim != 2 || p.SOLID || p.PLASTIC) return false;
    if (p.n_materials < 1 || p.n_materials > 4) return false;
    for (int m = 0; m < p.n_materials; ++m)
        if (p.materials[m].eos != TJ_EOS_MIEGRUNEISEN || p.materials[m].phase != TJ_PHASE_FLUID) return false;
    return true;
}

static size_t smem_bytes(int M, int thinc)
{
    switch (M * 2 + (thinc ? 1 : 0)) {
        case 2: return Smem<1, false>::BYTES;
        case 3: return Smem<1, true>::BYTES;
        case 4: return Smem<2, false>::BYTES;
        case 5: return Smem<2, true>::BYTES;
        case 6: return Smem<3, false>::BYTES;
        case 7: return Smem<3, true>::BYTES;
        case 8: return Smem<4, false>::BYTES;
        default: return Smem<4, true>::BYTES;
    }
}

int mixed_alloc(MixedState& ms, const DevParams& DP, const std::vector<DevDomain>& doms, long long ntot,
                const long long* nftot, cudaStream_t st)
{
    (void)nftot;
    if (doms.size() != 1) return TJ_ERR_ARG;  // one 2-D domain
    MixedImpl* m = new MixedImpl();
    ms.impl = m;
    ms.allocated = true;
    const DevDomain& D = doms[0];
    m->M = DP.M;
    m->thinc = DP.thinc;
    MixP& P = m->P;
    std::memset(&P, 0, sizeof P);
    P.nx = D.n[0];
    P.ny = D.n[1];
    P.M = DP.M;
    P.thinc = DP.thinc;
    for (int d = 0; d < 2; ++d) {
        P.lo_bc[d] = DP.lo_bc[d];
        P.hi_bc[d] = DP.hi_bc[d];
        P.dx[d] = (float)D.dx[d];
    }
    P.beta = (float)DP.beta;
    P.cfl = DP.cfl;
    for (int k = 0; k < DP.M; ++k) {
        double G = DP.prm[k][0] - 1.0;
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
    const long long N = ntot;
    const int NW = 3 * DP.M + 7;
    for (int q = 0; q < 2; ++q) {
        if (cudaMalloc(&m->X[q], sizeof(float) * NW * N) != cudaSuccess) return TJ_ERR_CUDA;
        cudaMemsetAsync(m->X[q], 0, sizeof(float) * NW * N, st);
    }
    if (DP.thinc) {
        const long long nf[2] = {(long long)(P.nx + 1) * P.ny, (long long)P.nx * (P.ny + 1)};
        for (int q = 0; q < 2; ++q) {
            if (cudaMalloc(&m->starA[q], sizeof(float) * DP.M * N) != cudaSuccess) return TJ_ERR_CUDA;
            cudaMemsetAsync(m->starA[q], 0, sizeof(float) * DP.M * N, st);
            if (cudaMalloc(&m->urv[q], sizeof(float) * DP.M * N) != cudaSuccess) return TJ_ERR_CUDA;
            cudaMemsetAsync(m->urv[q], 0, sizeof(float) * DP.M * N, st);
            if (cudaMalloc(&m->urs[q], sizeof(int) * DP.M * N) != cudaSuccess) return TJ_ERR_CUDA;
            cudaMemsetAsync(m->urs[q], 0xFF, sizeof(int) * DP.M * N, st);
            for (int d = 0; d < 2; ++d) {
                if (cudaMalloc(&m->gstar[d][q], sizeof(float) * DP.M * nf[d]) != cudaSuccess) return TJ_ERR_CUDA;
                cudaMemsetAsync(m->gstar[d][q], 0, sizeof(float) * DP.M * nf[d], st);
            }
        }
    }
    for (int d = 0; d < 2; ++d) {
        const int n = d == 0 ? P.nx : P.ny;
        if (cudaMalloc(&m->bx[2 * d], sizeof(int) * n) != cudaSuccess) return TJ_ERR_CUDA;
        if (cudaMalloc(&m->bx[2 * d + 1], sizeof(int) * n) != cudaSuccess) return TJ_ERR_CUDA;
    }
    if (cudaMalloc(&m->ctr, sizeof(int)) != cudaSuccess) return TJ_ERR_CUDA;
    cudaMemsetAsync(m->ctr, 0, sizeof(int), st);
    if (cudaMalloc(&m->bad, sizeof(int)) != cudaSuccess) return TJ_ERR_CUDA;
    cudaMemsetAsync(m->bad, 0, sizeof(int), st);
    MixB& b = m->b;
    for (int q = 0; q < 2; ++q) {
        b.X[q] = m->X[q];
        b.starA[q] = m->starA[q];
        b.urv[q] = m->urv[q];
        b.urs[q] = m->urs[q];
        for (int d = 0; d < 2; ++d) b.gstar[d][q] = m->gstar[d][q];
    }
    b.bxlo[0] = m->bx[0];
    b.bxhi[0] = m->bx[1];
    b.bxlo[1] = m->bx[2];
    b.bxhi[1] = m->bx[3];
    b.stage_ctr = m->ctr;
    b.N = N;
    b.scal = nullptr;
    // one-box default box tables
    std::vector<std::vector<int>> one{{0, 0, 0, P.nx - 1, P.ny - 1, 0}};
    return mixed_set_boxes(ms, DP, doms, one, st);
}

void mixed_free(MixedState& ms)
{
    MixedImpl* m = (MixedImpl*)ms.impl;
    if (!m) return;
    float* fs[] = {m->X[0], m->X[1], m->starA[0], m->starA[1], m->urv[0], m->urv[1],
                   m->gstar[0][0], m->gstar[0][1], m->gstar[1][0], m->gstar[1][1]};
    for (float* p : fs)
        if (p) cudaFree(p);
    int* is[] = {m->urs[0], m->urs[1], m->bx[0], m->bx[1], m->bx[2], m->bx[3], m->ctr, m->bad};
    for (int* p : is)
        if (p) cudaFree(p);
    delete m;
    ms.impl = nullptr;
    ms.allocated = false;
}

int mixed_set_boxes(MixedState& ms, const DevParams& DP, const std::vector<DevDomain>& doms,
                    const std::vector<std::vector<int>>& boxes, cudaStream_t st)
{
    (void)DP;
    MixedImpl* m = (MixedImpl*)ms.impl;
    if (!m) return TJ_OK;
    const DevDomain& D = doms[0];
    const std::vector<int>& bl = boxes[0];
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
        cudaMemcpyAsync(m->bx[2 * d], lo[d].data(), sizeof(int) * D.n[d], cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(m->bx[2 * d + 1], hi[d].data(), sizeof(int) * D.n[d], cudaMemcpyHostToDevice, st);
    }
    const int* L = &bl[6 * (nb - 1)];
    m->P.last_box[0] = L[0];
    m->P.last_box[1] = L[1];
    m->P.last_box[2] = L[3];
    m->P.last_box[3] = L[4];
    cudaStreamSynchronize(st);
    return TJ_OK;
}

static int nblk(long long n) { return (int)std::min<long long>((n + 255) / 256, 152 * 8); }

int mixed_from_fp64(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st)
{
    MixedImpl* m = (MixedImpl*)ms.impl;
    m->b.scal = fb.scal;
    cudaMemsetAsync(m->bad, 0, sizeof(int), st);
    switch (m->M) {
        case 1: k_from_fp64<1><<<nblk(m->b.N), 256, 0, st>>>(DP, m->b, fb.A, m->bad); break;
        case 2: k_from_fp64<2><<<nblk(m->b.N), 256, 0, st>>>(DP, m->b, fb.A, m->bad); break;
        case 3: k_from_fp64<3><<<nblk(m->b.N), 256, 0, st>>>(DP, m->b, fb.A, m->bad); break;
        default: k_from_fp64<4><<<nblk(m->b.N), 256, 0, st>>>(DP, m->b, fb.A, m->bad); break;
    }
    int bad = 0;
    cudaMemcpyAsync(&bad, m->bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (bad) std::fprintf(stderr, "tenjin_gpu: mixed precision carries two velocity components; w was nonzero\n");
    return 1 + mixed_compute_dt(ms, DP, fb, st);
}

int mixed_to_fp64(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st)
{
    MixedImpl* m = (MixedImpl*)ms.impl;
    switch (m->M) {
        case 1: k_to_fp64<1><<<nblk(m->b.N), 256, 0, st>>>(DP, m->b, fb.A); break;
        case 2: k_to_fp64<2><<<nblk(m->b.N), 256, 0, st>>>(DP, m->b, fb.A); break;
        case 3: k_to_fp64<3><<<nblk(m->b.N), 256, 0, st>>>(DP, m->b, fb.A); break;
        default: k_to_fp64<4><<<nblk(m->b.N), 256, 0, st>>>(DP, m->b, fb.A); break;
    }
    return 1;
}

int mixed_compute_dt(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st)
{
    (void)DP;
    MixedImpl* m = (MixedImpl*)ms.impl;
    m->b.scal = fb.scal;
    k_reset_dtmin<<<1, 32, 0, st>>>(fb.scal);
    switch (m->M) {
        case 1: k_cfl_mixed<1><<<nblk(m->b.N), 256, 0, st>>>(m->P, m->b); break;
        case 2: k_cfl_mixed<2><<<nblk(m->b.N), 256, 0, st>>>(m->P, m->b); break;
        case 3: k_cfl_mixed<3><<<nblk(m->b.N), 256, 0, st>>>(m->P, m->b); break;
        default: k_cfl_mixed<4><<<nblk(m->b.N), 256, 0, st>>>(m->P, m->b); break;
    }
    return 1;
}

template <int M, bool THINC>
static void launch_stage(MixedImpl* m, int stage, cudaStream_t st)
{
    static bool attr = false;
    const size_t sm = Smem<M, THINC>::BYTES;
    if (!attr) {
        cudaFuncSetAttribute(k_stage2d<M, THINC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = true;
    }
    dim3 grid((m->P.nx + MT - 1) / MT, (m->P.ny + MT - 1) / MT);
    k_stage2d<M, THINC><<<grid, NTH, sm, st>>>(m->P, m->b, stage);
}

static void stage_dispatch(MixedImpl* m, int stage, cudaStream_t st)
{
    switch (m->M * 2 + (m->thinc ? 1 : 0)) {
        case 2: launch_stage<1, false>(m, stage, st); break;
        case 3: launch_stage<1, true>(m, stage, st); break;
        case 4: launch_stage<2, false>(m, stage, st); break;
        case 5: launch_stage<2, true>(m, stage, st); break;
        case 6: launch_stage<3, false>(m, stage, st); break;
        case 7: launch_stage<3, true>(m, stage, st); break;
        case 8: launch_stage<4, false>(m, stage, st); break;
        default: launch_stage<4, true>(m, stage, st); break;
    }
}

int mixed_step(MixedState& ms, const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st, Prof* pr)
{
    MixedImpl* m = (MixedImpl*)ms.impl;
    m->b.scal = fb.scal;
    int n = 0;
    n += fp64_dt_finalize(DP, fb, 1, st);
    for (int stage = 0; stage < 2; ++stage) {
        if (pr) pr->begin("tj_stage_mixed", st);
        stage_dispatch(m, stage, st);
        if (pr) pr->end("tj_stage_mixed", st);
        k_stage_ctr_inc<<<1, 32, 0, st>>>(m->ctr, fb.scal);
        n += 2;
    }
    n += fp64_step_end(fb, st);
    return n;
}

int mixed_launches_per_step(const DevParams& DP)
{
    (void)DP;
    return 6;
}


}  // namespace tj
