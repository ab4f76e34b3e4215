// Device-side physics of the Tenjin per-timestep update: equations of state,
// primitive/conservative closures, sound speed, Hencky strain, stress and the
// 3x3 algebra. One source for two working types: the parameter block PT
// (DevParams: binary64; DevParams32: binary32) fixes R = PT::real. Every
// expression keeps the evaluation order of the reference (file:line
// citations), so that the binary64 instance, compiled with -fmad=false,
// reproduces the reference's results bit for bit; literals are written R(x),
// which is x itself in binary64.
#pragma once

#include <type_traits>

#include <cstdint>

#include "tj_math.cuh"
#include "tj_types.h"

namespace tj {

// ---------------------------------------------------------------------------
// Per-cell state in registers (the reference's Cell view, cell.h:42-84).
// ---------------------------------------------------------------------------
// Equality of bit patterns (the repeated cleanUpAlpha's convergence test).
__device__ __forceinline__ bool same_bits(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b);
}
__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_int(a) == __float_as_int(b); }

template <typename R>
struct CellT {
    R alpha[TJ_MAX_MAT], arho[TJ_MAX_MAT], rhok[TJ_MAX_MAT];
    R rho, rhou[3], vel[3], E, p, a;
    R sigma[9];
    R V[9], devH[9], hj2;
    R eps[TJ_MAX_MAT], are[TJ_MAX_MAT];
    R Elo;  // binary32 state: the low word of the compensated total energy
    R lam, arl, rm0, rm1;  // MixtureEOS (material 0): lambda, alphaRhoLambda, rhomix rows 0 and 1
};
using CellS = CellT<double>;

template <typename R>
struct ECellT {
    R alpha, arho, rhok, p, hj2;
    R lam, rm0, rm1;  // MixtureEOS only
};
using ECell = ECellT<double>;

template <typename R>
__device__ __forceinline__ ECellT<R> ecell_of(const CellT<R>& c, int m)
{
    ECellT<R> e;
    e.alpha = c.alpha[m];
    e.arho = c.arho[m];
    e.rhok = c.rhok[m];
    e.p = c.p;
    e.hj2 = c.hj2;
    e.lam = c.lam;
    e.rm0 = c.rm0;
    e.rm1 = c.rm1;
    return e;
}

// ---------------------------------------------------------------------------
// Equations of state (equationofstate.cpp).
// Parameter vectors as getMaterialParameters builds them (initialise.cpp:125-235).
// ---------------------------------------------------------------------------
template <typename PT>
__device__ __forceinline__ typename PT::real gam(const PT& P, int m)
{
    using R = typename PT::real;
    return P.prm[m][0] - R(1.0);
}

// MixtureEOS (equationofstate.cpp:117-396): two stiffened gases, parameters
// [gamma, pref, eref, CV] x 2, blended by the mass fraction lambda. The
// effective gamma - 1 of :175 and :224.
template <typename PT>
__device__ __forceinline__ typename PT::real mix_gamma_term(const PT& P, int m, typename PT::real lam)
{
    using R = typename PT::real;
    const R* q = P.prm[m];
    return (lam * q[0] * q[3] + (R(1.0) - lam) * q[4] * q[7]) / (lam * q[3] + (R(1.0) - lam) * q[7]) - R(1.0);
}

template <typename PT>
__device__ inline typename PT::real eos_e_cold(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    const R* q = P.prm[m];
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return q[2] * e.arho;  // equationofstate.cpp:37-40
        case TJ_EOS_MIXTURE: return e.lam * (q[2] * e.arho) + (R(1.0) - e.lam) * (q[6] * e.arho);  // :161-165
        case TJ_EOS_ROMENSKII: {                         // :418-423
            R a = q[6], K0 = q[5], r0 = q[4], x = e.rhok / r0;
            return e.arho * (((K0 / (R(2.0) * r0 * a * a)) * (tjm_pow(x, a) - R(1.0))) * (tjm_pow(x, a) - R(1.0)));
        }
        case TJ_EOS_WILKINS: {  // :519-524
            R r0 = q[4], x = e.rhok / r0;
            return e.arho * ((q[5] + q[6] * x * x + q[7] * x + q[8] / x - q[9] * tjm_log(x)) / r0);
        }
        default: {  // Hugoniot reference curve (copper; no reference class)
            R r0 = q[4], c0 = q[5], sl = q[6];
            R et = R(1.0) - r0 / e.rhok, dd = R(1.0) - sl * et;
            R ph = r0 * c0 * c0 * et / (dd * dd);
            return e.arho * (ph * et / (R(2.0) * r0));
        }
    }
}

template <typename PT>
__device__ inline typename PT::real eos_p_cold(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    const R* q = P.prm[m];
    R G = gam(P, m);
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return q[1] * e.alpha / G;  // :42-45
        case TJ_EOS_MIXTURE:                                  // :167-171
            return (q[1] * e.alpha / (q[0] - R(1.0))) * e.lam * e.rhok / (e.rm0) +
                   (q[5] * e.alpha / (q[4] - R(1.0))) * (R(1.0) - e.lam) * e.rhok / (e.rm1);
        case TJ_EOS_ROMENSKII: {                              // :425-430
            R a = q[6], K0 = q[5], r0 = q[4], x = e.rhok / r0;
            return (e.alpha / G) * ((K0 / a) * tjm_pow(x, a + R(1.0)) * (tjm_pow(x, a) - R(1.0)));
        }
        case TJ_EOS_WILKINS: {  // :526-531
            R r0 = q[4], x = e.rhok / r0;
            return (e.alpha / G) * ((R(2.0) * q[6] * x * x * x + q[7] * x * x - q[8] - q[9] * x));
        }
        default: {
            R r0 = q[4], c0 = q[5], sl = q[6];
            R et = R(1.0) - r0 / e.rhok, dd = R(1.0) - sl * et;
            R ph = r0 * c0 * c0 * et / (dd * dd);
            return (e.alpha / G) * ph;
        }
    }
}

template <typename PT>
__device__ inline typename PT::real eos_G(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    const R* q = P.prm[m];
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return R(0.0) * e.alpha;                           // :81-84
        case TJ_EOS_MIXTURE: return R(0.0);                                          // :146-149
        case TJ_EOS_ROMENSKII: return q[8] * tjm_pow((e.rhok / q[4]), q[7] + R(1.0));  // :437-440
        case TJ_EOS_WILKINS: return q[10];                                           // :538-541
        default: return q[7];
    }
}

template <typename PT>
__device__ inline typename PT::real eos_dGdrho(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    const R* q = P.prm[m];
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return R(0.0) * e.alpha;
        case TJ_EOS_ROMENSKII: return q[8] * (q[7] + R(1.0)) * tjm_pow((e.rhok / q[4]), q[7]) / q[4];  // :442-445
        default: return R(0.0);
    }
}

template <typename PT>
__device__ inline typename PT::real eos_dG2drho2(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    const R* q = P.prm[m];
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return R(0.0) * e.alpha;
        case TJ_EOS_ROMENSKII:  // :447-450
            return q[8] * (q[7] + R(1.0)) * (q[7]) * tjm_pow((e.rhok / q[4]), q[7] - R(1.0)) / (q[4] * q[4]);
        default: return R(0.0);
    }
}

template <typename PT>
__device__ inline typename PT::real eos_e_shear(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return R(0.0) * e.alpha;  // :101-104
        case TJ_EOS_MIXTURE: return R(0.0);                 // :136-139
        case TJ_EOS_HUGONIOT: return e.alpha * (P.prm[m][7] * e.hj2);
        default: return e.alpha * (eos_G(P, m, e) * e.hj2);  // :457-460, :558-561
    }
}

template <typename PT>
__device__ inline typename PT::real eos_p_shear(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    R G = gam(P, m);
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return R(0.0) * e.alpha;  // :106-109
        case TJ_EOS_MIXTURE: return R(0.0);                 // :141-144
        case TJ_EOS_HUGONIOT: return (e.alpha / G) * ((e.rhok * R(0.0) - P.prm[m][7]) * e.hj2);
        default: return (e.alpha / G) * ((e.rhok * eos_dGdrho(P, m, e) - eos_G(P, m, e)) * e.hj2);  // :462-465
    }
}

template <typename PT>
__device__ __forceinline__ typename PT::real eos_invG(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    if (P.eos[m] == TJ_EOS_MIXTURE) return e.alpha / mix_gamma_term(P, m, e.lam);  // :173-178
    return e.alpha / gam(P, m);
}

// xi (equationofstate.cpp:72-75, 222-225)
template <typename PT>
__device__ __forceinline__ typename PT::real eos_xi(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    if (P.eos[m] == TJ_EOS_MIXTURE) return R(1.0) / mix_gamma_term(P, m, e.lam);
    return R(1.0) / gam(P, m);
}

// Sound-speed contribution c^2_m (getSoundSpeedContribution).
template <typename PT>
__device__ inline typename PT::real eos_c2(const PT& P, int m, const ECellT<typename PT::real>& e)
{
    using R = typename PT::real;
    const R* q = P.prm[m];
    R G = gam(P, m);
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return e.p * (G + R(1.0)) / e.rhok - q[1] / e.rhok;  // :61-64
        case TJ_EOS_MIXTURE: {  // mixtureSoundSpeed (:208-220)
            const R G1 = q[0] - R(1.0), G2 = q[4] - R(1.0);
            R dedrho = (e.lam) * ((q[1] - e.p) / (G1 * e.rhok * e.rhok));
            dedrho += (R(1.0) - e.lam) * ((q[5] - e.p) / (G2 * e.rhok * e.rhok));
            return (e.p / (e.rhok * e.rhok) - dedrho) / (e.lam / (e.rm0 * G1) + (R(1.0) - e.lam) / (e.rm1 * G2));
        }
        case TJ_EOS_ROMENSKII: {                                                       // :432-435
            R a = q[6], K0 = q[5], r0 = q[4], x = e.rhok / r0;
            R dpc = (K0 / (a * r0)) * tjm_pow(x, a) * ((R(2.0) * a + R(1.0)) * tjm_pow(x, a) - (a + R(1.0)));
            R dps = e.rhok * eos_dG2drho2(P, m, e) * e.hj2;
            return (e.p * (G + R(1.0)) - (eos_p_cold(P, m, e) + eos_p_shear(P, m, e)) * (G + R(1.0))) / e.rhok + dpc +
                   dps + R(4.0 / 3.0) * eos_G(P, m, e) / e.rhok;
        }
        case TJ_EOS_WILKINS: {  // :533-536
            R r0 = q[4], x = e.rhok / r0;
            R dpc = (R(6.0) * q[6] * x * x + R(2.0) * q[7] * x - q[9]) / r0;
            R dps = e.rhok * eos_dG2drho2(P, m, e) * e.hj2;
            return (e.p * (G + R(1.0)) - (eos_p_cold(P, m, e) + eos_p_shear(P, m, e)) * (G + R(1.0))) / e.rhok + dpc +
                   dps + R(4.0 / 3.0) * eos_G(P, m, e) / e.rhok;
        }
        default: {  // Mie-Gruneisen sound speed on the Hugoniot reference curve
            R r0 = q[4], c0 = q[5], sl = q[6], G0 = q[7];
            R rho = e.rhok, et = R(1.0) - r0 / rho, dd = R(1.0) - sl * et;
            R ph = r0 * c0 * c0 * et / (dd * dd);
            R dph = r0 * c0 * c0 * (R(1.0) + sl * et) / (dd * dd * dd);
            R detadrho = r0 / (rho * rho);
            R dp = dph * detadrho;
            R de = (ph + et * dph) / (R(2.0) * r0) * detadrho;
            return dp - G * rho * de + (e.p * (G + R(1.0)) - ph) / rho + R(4.0 / 3.0) * G0 / rho;
        }
    }
}

// ---------------------------------------------------------------------------
// 3x3 algebra (tensor.cpp).
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R det2(R a, R b, R c, R d)
{
    return a * d - b * c;
}

// Cofactor expansion along the first row (tensor.cpp:296-333).
template <typename R>
__device__ inline R det3(const R* M)
{
    R det = R(0.0);
    det += (R(1.0) * M[0]) * det2(M[4], M[5], M[7], M[8]);
    det += (R(-1.0) * M[1]) * det2(M[3], M[5], M[6], M[8]);
    det += (R(1.0) * M[2]) * det2(M[3], M[4], M[6], M[7]);
    return det;
}

// Transposed cofactors over the determinant (tensor.cpp:187-233).
template <typename R>
__device__ inline void invert3(const R* M, R* Minv)
{
    R D = det3(M);
    R c00 = det2(M[4], M[5], M[7], M[8]), c01 = R(-1.0) * det2(M[3], M[5], M[6], M[8]),
      c02 = det2(M[3], M[4], M[6], M[7]);
    R c10 = R(-1.0) * det2(M[1], M[2], M[7], M[8]), c11 = det2(M[0], M[2], M[6], M[8]),
      c12 = R(-1.0) * det2(M[0], M[1], M[6], M[7]);
    R c20 = det2(M[1], M[2], M[4], M[5]), c21 = R(-1.0) * det2(M[0], M[2], M[3], M[5]),
      c22 = det2(M[0], M[1], M[3], M[4]);
    Minv[0] = c00 / D; Minv[1] = c10 / D; Minv[2] = c20 / D;
    Minv[3] = c01 / D; Minv[4] = c11 / D; Minv[5] = c21 / D;
    Minv[6] = c02 / D; Minv[7] = c12 / D; Minv[8] = c22 / D;
}

// Row-major product, k summed innermost in increasing order (the reference
// BLAS order for each element, tensor.cpp:81-115).
template <typename R>
__device__ inline void mm3(const R* A, const R* B, R* C)
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            R s = R(0.0);
            s += A[i * 3 + 0] * B[0 * 3 + j];
            s += A[i * 3 + 1] * B[1 * 3 + j];
            s += A[i * 3 + 2] * B[2 * 3 + j];
            C[i * 3 + j] = s;
        }
}
template <typename R>
__device__ inline void mmT3(const R* A, const R* B, R* C)  // A B^T
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            R s = R(0.0);
            s += A[i * 3 + 0] * B[j * 3 + 0];
            s += A[i * 3 + 1] * B[j * 3 + 1];
            s += A[i * 3 + 2] * B[j * 3 + 2];
            C[i * 3 + j] = s;
        }
}
template <typename R>
__device__ __forceinline__ R trace3(const R* M)
{
    R t = R(0.0);
    t += M[0];
    t += M[4];
    t += M[8];
    return t;
}

// Symmetric 3x3 eigendecomposition by cyclic Jacobi rotations (Golub & Van
// Loan, Matrix Computations, sec. 8.5). w decreasing; q holds the
// eigenvectors as columns. Bounded at 50 sweeps.
template <typename R>
__device__ inline void sym3_eig(const R* a_in, R* w, R* q)
{
    R a[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) a[i] = a_in[i];
#pragma unroll
    for (int i = 0; i < 9; ++i) q[i] = (i % 4 == 0) ? R(1.0) : R(0.0);
    for (int sweep = 0; sweep < 50; ++sweep) {
        R off = fabs(a[1]) + fabs(a[2]) + fabs(a[5]);
        if (off == R(0.0)) break;
#pragma unroll
        for (int pr = 0; pr < 3; ++pr) {
            const int p = pr < 2 ? 0 : 1, r = pr == 0 ? 1 : 2;
            R apr = a[p * 3 + r];
            if (apr == R(0.0)) continue;
            R app = a[p * 3 + p], arr = a[r * 3 + r];
            R theta = (arr - app) / (R(2.0) * apr);
            R t = (theta >= R(0.0) ? R(1.0) : R(-1.0)) / (fabs(theta) + sqrt(theta * theta + R(1.0)));
            R c = R(1.0) / sqrt(t * t + R(1.0));
            R s = t * c;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                R akp = a[k * 3 + p], akr = a[k * 3 + r];
                a[k * 3 + p] = c * akp - s * akr;
                a[k * 3 + r] = s * akp + c * akr;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                R apk = a[p * 3 + k], ark = a[r * 3 + k];
                a[p * 3 + k] = c * apk - s * ark;
                a[r * 3 + k] = s * apk + c * ark;
            }
            a[p * 3 + r] = R(0.0);
            a[r * 3 + p] = R(0.0);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                R qkp = q[k * 3 + p], qkr = q[k * 3 + r];
                q[k * 3 + p] = c * qkp - s * qkr;
                q[k * 3 + r] = s * qkp + c * qkr;
            }
        }
    }
    // decreasing order by an exchange sort on positions (0,1,2) that swaps
    // the eigenvalues and their columns themselves (every index is a
    // compile-time constant, so nothing leaves the registers)
    R d[3] = {a[0], a[4], a[8]};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i + 1; j < 3; ++j)
            if (d[j] > d[i]) {
                const R t = d[i];
                d[i] = d[j];
                d[j] = t;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const R u = q[r * 3 + i];
                    q[r * 3 + i] = q[r * 3 + j];
                    q[r * 3 + j] = u;
                }
            }
#pragma unroll
    for (int c = 0; c < 3; ++c) w[c] = d[c];
}

// matrixSquareRoot (tensor.cpp:452-475): L S^(1/2) RT with L = Q, RT = Q^T.
template <typename R>
__device__ inline void sqrtm3(const R* A, R* Rm)
{
    R w[3], q[9], L[9], RT[9], S[9], tmp[9];
    sym3_eig(A, w, q);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            L[i * 3 + j] = q[i * 3 + j];
            RT[i * 3 + j] = q[j * 3 + i];
            S[i * 3 + j] = sqrt(w[i]) * (R)(i == j);
        }
    mm3(L, S, tmp);
    mm3(tmp, RT, Rm);
}

// ---------------------------------------------------------------------------
// BoxAccessCellArray per-cell operations (boxaccesscellarray.cpp).
// ---------------------------------------------------------------------------
template <typename PT>
__device__ inline typename PT::real eff_invG(const PT& P, const CellT<typename PT::real>& c)  // :218-228
{
    using R = typename PT::real;
    R tot = R(0.0);
    for (int m = 0; m < P.M; ++m) tot += eos_invG(P, m, ecell_of(c, m));
    return tot;
}
template <typename PT>
__device__ inline typename PT::real eff_e_nonthermal(const PT& P, const CellT<typename PT::real>& c)  // :230-240
{
    using R = typename PT::real;
    R tot = R(0.0);
    for (int m = 0; m < P.M; ++m) {
        ECellT<R> e = ecell_of(c, m);
        tot += (eos_e_cold(P, m, e) + eos_e_shear(P, m, e));
    }
    return tot;
}
template <typename PT>
__device__ inline typename PT::real eff_p_nonthermal(const PT& P, const CellT<typename PT::real>& c)  // :242-252
{
    using R = typename PT::real;
    R tot = R(0.0);
    for (int m = 0; m < P.M; ++m) {
        ECellT<R> e = ecell_of(c, m);
        tot += eos_p_cold(P, m, e) + eos_p_shear(P, m, e);
    }
    return tot;
}

// getDeviatoricHenckyStrain + getHenckyJ2 (:326-380); solids only.
template <typename PT>
__device__ inline void hencky(const PT& P, CellT<typename PT::real>& c)
{
    using R = typename PT::real;
    if (!P.any_solid) return;
    R B[9], Binv[9], prod[9];
    mmT3(c.V, c.V, B);
    invert3(B, Binv);
#pragma unroll
    for (int q = 0; q < 9; ++q) c.devH[q] = R(0.5) * R(0.5) * (B[q] - Binv[q]);
    mmT3(c.devH, c.devH, prod);
    c.hj2 = trace3(prod);
}

// stressTensor (:176-216)
template <typename PT>
__device__ inline void stress(const PT& P, CellT<typename PT::real>& c)
{
    using R = typename PT::real;
    R Gt = R(0.0);
    int solid = 0;
    for (int m = 0; m < P.M; ++m)
        if (P.phase[m] == TJ_PHASE_SOLID) {
            ECellT<R> e = ecell_of(c, m);
            solid = 1;
            Gt += eos_G(P, m, e) * (eos_invG(P, m, e));
        }
    Gt = Gt / eff_invG(P, c);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            R dl = (R)(r == q);
            c.sigma[3 * r + q] = solid ? (-c.p * dl + R(2.0) * Gt * c.devH[3 * r + q]) : (-c.p * dl);
        }
}

// MixtureEOS root finding (equationofstate.cpp:238-376) for material 0, in
// binary64: the mixture densities at which the two components' temperatures
// (p - pref)/(rho Gamma CV) agree, by bisection of rhomix_0 on
// [lambda rho_k + 1e-10, 1e6] to a relative width of 1e-7. Returns
// TJ_ERR_ROOT where the reference prints and exits (no sign change over the
// bracket), and after kMaxBisect halvings (the reference loops on; the width
// test passes after about 60 at most).
constexpr int kMaxBisect = 200;

__device__ __forceinline__ double mix_rhob(const CellT<double>& c, double rhoa)  // rhobFunc (:243-246)
{
    return (1.0 - c.lam) / (1.0 / c.rhok[0] - c.lam / rhoa);
}

__device__ __forceinline__ int sgn_d(double v) { return (0.0 < v) - (v < 0.0); }

template <typename PD>
__device__ inline double mix_bisect_f(const PD& P, CellT<double>& c, double rho_try, double ke)  // :262-272
{
    c.rm0 = rho_try;
    c.rm1 = mix_rhob(c, rho_try);
    const double p = (c.E - ke - eff_e_nonthermal(P, c) + eff_p_nonthermal(P, c)) / (eff_invG(P, c));
    const double* q = P.prm[0];
    // pressureFunction (:251-260)
    return ((p - q[1]) / (c.rm0 * (q[0] - 1.0) * q[3])) - ((p - q[5]) / (c.rm1 * (q[4] - 1.0) * q[7]));
}

template <typename PD>
__device__ inline int mix_root_find(const PD& P, CellT<double>& c, double ke)
{
    const double* q = P.prm[0];
    const double lam = c.lam, rk = c.rhok[0];
    if (q[1] == 0.0 && q[5] == 0.0) {
        c.rm0 = rk * (lam + (1.0 - lam) * ((q[4] - 1.0) * q[7]) / ((q[0] - 1.0) * q[3]));
        c.rm1 = mix_rhob(c, c.rm0);
        return 0;
    }
    if (lam > 1.0 - 1E-3) {
        c.rm0 = rk;
        c.rm1 = rk;
        return 0;
    } else if (lam < 1E-3) {
        c.rm1 = rk;
        c.rm0 = rk;
        return 0;
    }
    double A = lam * rk + 1E-10, B = 1000000.0;
    double mid = 0.5 * (A + B);
    if (fabs(mix_bisect_f(P, c, A, ke)) <= 1E-4) {
        c.rm0 = A;
        c.rm1 = mix_rhob(c, c.rm0);
        return 0;
    } else if (fabs(mix_bisect_f(P, c, B, ke)) <= 1E-4) {
        c.rm0 = B;
        c.rm1 = mix_rhob(c, c.rm0);
        return 0;
    }
    if (sgn_d(mix_bisect_f(P, c, A, ke)) == sgn_d(mix_bisect_f(P, c, B, ke))) return TJ_ERR_ROOT;
    for (int n = 0; n < kMaxBisect; ++n) {
        if (sgn_d(mix_bisect_f(P, c, mid, ke)) == sgn_d(mix_bisect_f(P, c, A, ke))) A = mid;
        else B = mid;
        mid = 0.5 * (A + B);
        if (fabs(A - B) / (A + B) < 1E-7) {
            c.rm0 = mid;
            c.rm1 = mix_rhob(c, c.rm0);
            return 0;
        }
    }
    return TJ_ERR_ROOT;
}

// The non-thermal energy, non-thermal pressure and alpha/Gamma terms of one
// material for the binary64 pressure closure of a binary32 cell: the
// formulas of eos_e_cold + eos_e_shear, eos_p_cold + eos_p_shear and
// eos_invG, with each quotient formed once and the constant ones taken from
// the precomputed reciprocals (a stiffened gas: no division instead of two,
// the Hugoniot curve: two instead of eight); other EOS go through the general
// functions.
template <typename P32>
__device__ __forceinline__ void closure_terms64(const P32& P, int m, const ECellT<double>& e, double& ent, double& pnt,
                                       double& ig)
{
    const double* q = P.d.prm[m];
    switch (P.d.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: {
            const double aG = e.alpha * P.rG[m];
            ent += q[2] * e.arho;
            pnt += q[1] * aG;
            ig += aG;
            return;
        }
        case TJ_EOS_HUGONIOT: {
            const double aG = e.alpha * P.rG[m];
            const double r0 = q[4], c0 = q[5], sl = q[6];
            const double et = 1.0 - r0 / e.rhok, dd = 1.0 - sl * et;
            const double ph = r0 * c0 * c0 * et / (dd * dd);
            ent += e.arho * (ph * et * P.rR0h[m]) + e.alpha * (q[7] * e.hj2);
            pnt += aG * ph - aG * (q[7] * e.hj2);
            ig += aG;
            return;
        }
        default:
            ent += eos_e_cold(P.d, m, e) + eos_e_shear(P.d, m, e);
            pnt += eos_p_cold(P.d, m, e) + eos_p_shear(P.d, m, e);
            ig += eos_invG(P.d, m, e);
    }
}

// (sh, sl) += b: the rounding error of sh + b (Knuth's two-sum, every
// operation rounded to nearest) is added to the low word.
__device__ __forceinline__ void acc_pair32(float& sh, float& sl, float b)
{
    const float s = __fadd_rn(sh, b);
    const float bb = __fsub_rn(s, sh);
    sl = __fadd_rn(sl, __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
    sh = s;
}

// conservativeToPrimitive (:67-122). Returns 0, or TJ_ERR_ROOT from the
// mixture closure.
template <typename PT>
__device__ __forceinline__ int c2p(const PT& P, CellT<typename PT::real>& c)
{
    using R = typename PT::real;
    int err = 0;
    c.rho = 0;
    for (int m = 0; m < P.M; ++m) {
        c.rhok[m] = c.arho[m] / c.alpha[m];
        c.rho += c.arho[m];
        if (P.plastic && P.phase[m] == TJ_PHASE_SOLID) c.eps[m] = c.are[m] / c.arho[m];
    }
    hencky(P, c);
    R ke = R(0.0);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        c.vel[r] = c.rhou[r] / c.rho;
        ke += R(0.5) * c.rho * c.vel[r] * c.vel[r];
    }
    if constexpr (sizeof(R) == 4) {
        if (P.M == 1 && !P.nmix) {
            // one material: no interface whose stiff cold terms cancel the
            // energy, so the closure stays binary32, with the numerator
            // E + Elo - KE - e_cold + p_cold summed without rounding error
            // into an unevaluated pair (error-free sums)
            const R ent = eff_e_nonthermal(P, c), pnt = eff_p_nonthermal(P, c), ig = eff_invG(P, c);
            R sh = c.E, sl = c.Elo;
            acc_pair32(sh, sl, -ke);
            acc_pair32(sh, sl, -ent);
            acc_pair32(sh, sl, pnt);
            c.p = __fadd_rn(sh, sl) / ig;
            stress(P, c);
            return err;
        }
        // binary32 state with several materials: the closure of the pressure
        // (and of the mixture densities) in binary64, from the compensated
        // energy (E, Elo) and binary64 cold terms
        double rho = 0.0, ent = 0.0, pnt = 0.0, ig = 0.0;
        for (int m = 0; m < P.M; ++m) rho += (double)c.arho[m];
        const double ru0 = c.rhou[0], ru1 = c.rhou[1], ru2 = c.rhou[2];
        const double ked = 0.5 * (ru0 * ru0 + ru1 * ru1 + ru2 * ru2) / rho;
        double lam = 0.0, rm0 = 0.0, rm1 = 0.0;
        if (P.nmix) {
            lam = (double)c.arl / (double)c.arho[0];
            CellT<double> cd;
            for (int m = 0; m < P.M; ++m) {
                cd.alpha[m] = c.alpha[m];
                cd.arho[m] = c.arho[m];
                cd.rhok[m] = c.rhok[m];
            }
            cd.hj2 = c.hj2;
            cd.p = 0.0;
            cd.E = (double)c.E + (double)c.Elo;
            cd.lam = lam;
            cd.rm0 = c.rm0;
            cd.rm1 = c.rm1;
            err = mix_root_find(P.d, cd, ked);
            rm0 = cd.rm0;
            rm1 = cd.rm1;
            c.lam = (R)lam;
            c.rm0 = (R)rm0;
            c.rm1 = (R)rm1;
        }
        for (int m = 0; m < P.M; ++m) {
            ECellT<double> e;
            e.alpha = c.alpha[m];
            e.arho = c.arho[m];
            e.rhok = c.rhok[m];
            e.p = 0.0;
            e.hj2 = c.hj2;
            e.lam = lam;
            e.rm0 = rm0;
            e.rm1 = rm1;
            if (P.nmix) {
                ent += eos_e_cold(P.d, m, e) + eos_e_shear(P.d, m, e);
                pnt += eos_p_cold(P.d, m, e) + eos_p_shear(P.d, m, e);
                ig += eos_invG(P.d, m, e);
            } else {
                closure_terms64(P, m, e, ent, pnt, ig);
            }
        }
        c.p = (R)(((double)c.E + (double)c.Elo - ked - ent + pnt) / ig);
    } else {
        if (P.nmix) {  // :104-113
            c.lam = c.arl / c.arho[0];
            // binary64 only: the tangent instance takes no mixtures
            if constexpr (std::is_same<R, double>::value) err = mix_root_find(P, c, ke);
        }
        c.p = (c.E - ke - eff_e_nonthermal(P, c) + eff_p_nonthermal(P, c)) / (eff_invG(P, c));
    }
    stress(P, c);
    return err;
}

// primitiveToConservative (:124-174)
template <typename PT>
__device__ inline void p2c(const PT& P, CellT<typename PT::real>& c)
{
    using R = typename PT::real;
    c.rho = 0;
    for (int m = 0; m < P.M; ++m) {
        c.arho[m] = c.alpha[m] * c.rhok[m];
        c.rho += c.arho[m];
        if (P.nmix && m == 0) {  // :142-147
            c.arl = c.lam * c.alpha[0] * c.rhok[0];
            // defineMixtureDensities (equationofstate.cpp:390-396)
            const R* q = P.prm[0];
            c.rm0 = c.rhok[0] * (c.lam + (R(1.0) - c.lam) * ((c.p - q[1]) / (c.p - q[5])) *
                                             ((q[7] * (q[4] - R(1.0))) / (q[3] * (q[0] - R(1.0)))));
            c.rm1 = (R(1.0) - c.lam) / (R(1.0) / c.rhok[0] - c.lam / c.rm0);
        }
        if (P.plastic && P.phase[m] == TJ_PHASE_SOLID) c.are[m] = c.eps[m] * c.arho[m];
    }
    hencky(P, c);
    R ke = R(0.0);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        c.rhou[r] = c.vel[r] * c.rho;
        ke += R(0.5) * c.rho * c.vel[r] * c.vel[r];
    }
    c.E = c.p * eff_invG(P, c) + eff_e_nonthermal(P, c) - eff_p_nonthermal(P, c) + ke;
    stress(P, c);
}

// getSoundSpeed (:254-285)
template <typename PT>
__device__ inline typename PT::real sound_speed(const PT& P, const CellT<typename PT::real>& c)
{
    using R = typename PT::real;
    R a = R(0.0), xit = R(0.0);
    for (int m = 0; m < P.M; ++m) {
        ECellT<R> e = ecell_of(c, m);
        R xi = eos_xi(P, m, e);
        R v = xi * eos_c2(P, m, e) * c.arho[m] / c.rho;
        a += (R(0.0) < v) ? v : R(0.0);
        xit += xi * c.alpha[m];
    }
    if (a <= R(0.0)) a = R(1E-6);
    return sqrt(a / xit);
}

// cleanUpAlpha on one cell (:530-599). Returns TJ_ERR_ALPHA on the
// reference's fatal conditions.
template <typename PT>
__device__ inline int cleanup_alpha(const PT& P, typename PT::real* alpha)
{
    using R = typename PT::real;
    R tot = R(0.0);
    int nan = 0;
    for (int m = 0; m < P.M; ++m) {
        R a = alpha[m];
        if (isnan(a)) {
            a = R(0.0);
            if (nan == 0) nan = m;
            else return TJ_ERR_ALPHA;
        } else if (a < R(0.0)) a = R(1E-6);
        else if (a > R(1.0)) a = R(1.0);
        alpha[m] = a;
        tot += a;
    }
    if (nan > 0) {
        alpha[nan] = R(1.0) - tot;
        tot += alpha[nan];
    }
    if (tot <= R(0.0)) return TJ_ERR_ALPHA;
    for (int m = 0; m < P.M; ++m) alpha[m] *= R(1.0) / tot;
    return 0;
}

// transverseWaveSpeed on a star state (:287-324).
template <typename PT>
__device__ inline typename PT::real transverse_speed(const PT& P, CellT<typename PT::real>& c)
{
    using R = typename PT::real;
    hencky(P, c);
    R b = R(0.0);
    for (int m = 0; m < P.M; ++m)
        if (P.phase[m] == TJ_PHASE_SOLID) {
            ECellT<R> e = ecell_of(c, m);
            b += eos_invG(P, m, e) * eos_G(P, m, e) / (c.rhok[m]);
        }
    if (isnan(b) || b < R(0.0)) b = R(0.0);
    R t = sqrt(b / eff_invG(P, c));
    if (isnan(t)) t = R(0.0);
    return t;
}

}  // namespace tj
