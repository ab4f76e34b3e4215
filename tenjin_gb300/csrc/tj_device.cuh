// Device-side physics of the Tenjin per-timestep update: equations of state,
// primitive/conservative closures, sound speed, Hencky strain, stress and the
// 3x3 algebra. Every expression keeps the evaluation order of the reference
// (file:line citations), so that the FP64 path reproduces the reference's
// results bit for bit; the translation units are compiled with -fmad=false.
#pragma once

#include <cstdint>

#include "tj_math.cuh"
#include "tj_types.h"

namespace tj {

// ---------------------------------------------------------------------------
// Per-cell state in registers (the reference's Cell view, cell.h:42-84).
// ---------------------------------------------------------------------------
struct CellS {
    double alpha[TJ_MAX_MAT], arho[TJ_MAX_MAT], rhok[TJ_MAX_MAT];
    double rho, rhou[3], vel[3], E, p, a;
    double sigma[9];
    double V[9], devH[9], hj2;
    double eps[TJ_MAX_MAT], are[TJ_MAX_MAT];
};

struct ECell {
    double alpha, arho, rhok, p, hj2;
};

__device__ __forceinline__ ECell ecell_of(const CellS& c, int m)
{
    ECell e;
    e.alpha = c.alpha[m];
    e.arho = c.arho[m];
    e.rhok = c.rhok[m];
    e.p = c.p;
    e.hj2 = c.hj2;
    return e;
}

// ---------------------------------------------------------------------------
// Equations of state (equationofstate.cpp).
// Parameter vectors as getMaterialParameters builds them (initialise.cpp:125-235).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double gam(const DevParams& P, int m) { return P.prm[m][0] - 1.0; }

__device__ inline double eos_e_cold(const DevParams& P, int m, const ECell& e)
{
    const double* q = P.prm[m];
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return q[2] * e.arho;  // equationofstate.cpp:37-40
        case TJ_EOS_ROMENSKII: {                         // :418-423
            double a = q[6], K0 = q[5], r0 = q[4], x = e.rhok / r0;
            return e.arho * (((K0 / (2.0 * r0 * a * a)) * (tjm_pow(x, a) - 1.0)) * (tjm_pow(x, a) - 1.0));
        }
        case TJ_EOS_WILKINS: {  // :519-524
            double r0 = q[4], x = e.rhok / r0;
            return e.arho * ((q[5] + q[6] * x * x + q[7] * x + q[8] / x - q[9] * tjm_log(x)) / r0);
        }
        default: {  // Hugoniot reference curve (copper; no reference class)
            double r0 = q[4], c0 = q[5], sl = q[6];
            double et = 1.0 - r0 / e.rhok, dd = 1.0 - sl * et;
            double ph = r0 * c0 * c0 * et / (dd * dd);
            return e.arho * (ph * et / (2.0 * r0));
        }
    }
}

__device__ inline double eos_p_cold(const DevParams& P, int m, const ECell& e)
{
    const double* q = P.prm[m];
    double G = gam(P, m);
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return q[1] * e.alpha / G;  // :42-45
        case TJ_EOS_ROMENSKII: {                              // :425-430
            double a = q[6], K0 = q[5], r0 = q[4], x = e.rhok / r0;
            return (e.alpha / G) * ((K0 / a) * tjm_pow(x, a + 1.0) * (tjm_pow(x, a) - 1.0));
        }
        case TJ_EOS_WILKINS: {  // :526-531
            double r0 = q[4], x = e.rhok / r0;
            return (e.alpha / G) * ((2.0 * q[6] * x * x * x + q[7] * x * x - q[8] - q[9] * x));
        }
        default: {
            double r0 = q[4], c0 = q[5], sl = q[6];
            double et = 1.0 - r0 / e.rhok, dd = 1.0 - sl * et;
            double ph = r0 * c0 * c0 * et / (dd * dd);
            return (e.alpha / G) * ph;
        }
    }
}

__device__ inline double eos_G(const DevParams& P, int m, const ECell& e)
{
    const double* q = P.prm[m];
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return 0.0 * e.alpha;                  // :81-84
        case TJ_EOS_ROMENSKII: return q[8] * tjm_pow((e.rhok / q[4]), q[7] + 1.0);  // :437-440
        case TJ_EOS_WILKINS: return q[10];                               // :538-541
        default: return q[7];
    }
}

__device__ inline double eos_dGdrho(const DevParams& P, int m, const ECell& e)
{
    const double* q = P.prm[m];
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return 0.0 * e.alpha;
        case TJ_EOS_ROMENSKII: return q[8] * (q[7] + 1.0) * tjm_pow((e.rhok / q[4]), q[7]) / q[4];  // :442-445
        default: return 0.0;
    }
}

__device__ inline double eos_dG2drho2(const DevParams& P, int m, const ECell& e)
{
    const double* q = P.prm[m];
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return 0.0 * e.alpha;
        case TJ_EOS_ROMENSKII:  // :447-450
            return q[8] * (q[7] + 1.0) * (q[7]) * tjm_pow((e.rhok / q[4]), q[7] - 1.0) / (q[4] * q[4]);
        default: return 0.0;
    }
}

__device__ inline double eos_e_shear(const DevParams& P, int m, const ECell& e)
{
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return 0.0 * e.alpha;          // :101-104
        case TJ_EOS_HUGONIOT: return e.alpha * (P.prm[m][7] * e.hj2);
        default: return e.alpha * (eos_G(P, m, e) * e.hj2);      // :457-460, :558-561
    }
}

__device__ inline double eos_p_shear(const DevParams& P, int m, const ECell& e)
{
    double G = gam(P, m);
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return 0.0 * e.alpha;  // :106-109
        case TJ_EOS_HUGONIOT: return (e.alpha / G) * ((e.rhok * 0.0 - P.prm[m][7]) * e.hj2);
        default: return (e.alpha / G) * ((e.rhok * eos_dGdrho(P, m, e) - eos_G(P, m, e)) * e.hj2);  // :462-465
    }
}

__device__ __forceinline__ double eos_invG(const DevParams& P, int m, const ECell& e) { return e.alpha / gam(P, m); }

// Sound-speed contribution c^2_m (getSoundSpeedContribution).
__device__ inline double eos_c2(const DevParams& P, int m, const ECell& e)
{
    const double* q = P.prm[m];
    double G = gam(P, m);
    switch (P.eos[m]) {
        case TJ_EOS_MIEGRUNEISEN: return e.p * (G + 1.0) / e.rhok - q[1] / e.rhok;  // :61-64
        case TJ_EOS_ROMENSKII: {                                                    // :432-435
            double a = q[6], K0 = q[5], r0 = q[4], x = e.rhok / r0;
            double dpc = (K0 / (a * r0)) * tjm_pow(x, a) * ((2.0 * a + 1.0) * tjm_pow(x, a) - (a + 1.0));
            double dps = e.rhok * eos_dG2drho2(P, m, e) * e.hj2;
            return (e.p * (G + 1.0) - (eos_p_cold(P, m, e) + eos_p_shear(P, m, e)) * (G + 1.0)) / e.rhok + dpc + dps +
                   (4.0 / 3.0) * eos_G(P, m, e) / e.rhok;
        }
        case TJ_EOS_WILKINS: {  // :533-536
            double r0 = q[4], x = e.rhok / r0;
            double dpc = (6.0 * q[6] * x * x + 2.0 * q[7] * x - q[9]) / r0;
            double dps = e.rhok * eos_dG2drho2(P, m, e) * e.hj2;
            return (e.p * (G + 1.0) - (eos_p_cold(P, m, e) + eos_p_shear(P, m, e)) * (G + 1.0)) / e.rhok + dpc + dps +
                   (4.0 / 3.0) * eos_G(P, m, e) / e.rhok;
        }
        default: {  // Mie-Gruneisen sound speed on the Hugoniot reference curve
            double r0 = q[4], c0 = q[5], sl = q[6], G0 = q[7];
            double rho = e.rhok, et = 1.0 - r0 / rho, dd = 1.0 - sl * et;
            double ph = r0 * c0 * c0 * et / (dd * dd);
            double dph = r0 * c0 * c0 * (1.0 + sl * et) / (dd * dd * dd);
            double detadrho = r0 / (rho * rho);
            double dp = dph * detadrho;
            double de = (ph + et * dph) / (2.0 * r0) * detadrho;
            return dp - G * rho * de + (e.p * (G + 1.0) - ph) / rho + (4.0 / 3.0) * G0 / rho;
        }
    }
}

// ---------------------------------------------------------------------------
// 3x3 algebra (tensor.cpp).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double det2(double a, double b, double c, double d) { return a * d - b * c; }

// Cofactor expansion along the first row (tensor.cpp:296-333).
__device__ inline double det3(const double* M)
{
    double det = 0.0;
    det += (1.0 * M[0]) * det2(M[4], M[5], M[7], M[8]);
    det += (-1.0 * M[1]) * det2(M[3], M[5], M[6], M[8]);
    det += (1.0 * M[2]) * det2(M[3], M[4], M[6], M[7]);
    return det;
}

// Transposed cofactors over the determinant (tensor.cpp:187-233).
__device__ inline void invert3(const double* M, double* Minv)
{
    double D = det3(M);
    double c00 = det2(M[4], M[5], M[7], M[8]), c01 = -1.0 * det2(M[3], M[5], M[6], M[8]),
           c02 = det2(M[3], M[4], M[6], M[7]);
    double c10 = -1.0 * det2(M[1], M[2], M[7], M[8]), c11 = det2(M[0], M[2], M[6], M[8]),
           c12 = -1.0 * det2(M[0], M[1], M[6], M[7]);
    double c20 = det2(M[1], M[2], M[4], M[5]), c21 = -1.0 * det2(M[0], M[2], M[3], M[5]),
           c22 = det2(M[0], M[1], M[3], M[4]);
    Minv[0] = c00 / D; Minv[1] = c10 / D; Minv[2] = c20 / D;
    Minv[3] = c01 / D; Minv[4] = c11 / D; Minv[5] = c21 / D;
    Minv[6] = c02 / D; Minv[7] = c12 / D; Minv[8] = c22 / D;
}

// Row-major product, k summed innermost in increasing order (the reference
// BLAS order for each element, tensor.cpp:81-115).
__device__ inline void mm3(const double* A, const double* B, double* C)
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            s += A[i * 3 + 0] * B[0 * 3 + j];
            s += A[i * 3 + 1] * B[1 * 3 + j];
            s += A[i * 3 + 2] * B[2 * 3 + j];
            C[i * 3 + j] = s;
        }
}
__device__ inline void mmT3(const double* A, const double* B, double* C)  // A B^T
{
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            s += A[i * 3 + 0] * B[j * 3 + 0];
            s += A[i * 3 + 1] * B[j * 3 + 1];
            s += A[i * 3 + 2] * B[j * 3 + 2];
            C[i * 3 + j] = s;
        }
}
__device__ __forceinline__ double trace3(const double* M)
{
    double t = 0.0;
    t += M[0];
    t += M[4];
    t += M[8];
    return t;
}

// Symmetric 3x3 eigendecomposition by cyclic Jacobi rotations (Golub & Van
// Loan, Matrix Computations, sec. 8.5). w decreasing; q holds the
// eigenvectors as columns. Bounded at 50 sweeps.
__device__ inline void sym3_eig(const double* a_in, double* w, double* q)
{
    double a[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) a[i] = a_in[i];
#pragma unroll
    for (int i = 0; i < 9; ++i) q[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = fabs(a[1]) + fabs(a[2]) + fabs(a[5]);
        if (off == 0.0) break;
#pragma unroll
        for (int pr = 0; pr < 3; ++pr) {
            const int p = pr < 2 ? 0 : 1, r = pr == 0 ? 1 : 2;
            double apr = a[p * 3 + r];
            if (apr == 0.0) continue;
            double app = a[p * 3 + p], arr = a[r * 3 + r];
            double theta = (arr - app) / (2.0 * apr);
            double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            double c = 1.0 / sqrt(t * t + 1.0);
            double s = t * c;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double akp = a[k * 3 + p], akr = a[k * 3 + r];
                a[k * 3 + p] = c * akp - s * akr;
                a[k * 3 + r] = s * akp + c * akr;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double apk = a[p * 3 + k], ark = a[r * 3 + k];
                a[p * 3 + k] = c * apk - s * ark;
                a[r * 3 + k] = s * apk + c * ark;
            }
            a[p * 3 + r] = 0.0;
            a[r * 3 + p] = 0.0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double qkp = q[k * 3 + p], qkr = q[k * 3 + r];
                q[k * 3 + p] = c * qkp - s * qkr;
                q[k * 3 + r] = s * qkp + c * qkr;
            }
        }
    }
    int o0 = 0, o1 = 1, o2 = 2;
    double d[3] = {a[0], a[4], a[8]};
    // selection order identical to a stable exchange sort on (0,1,2)
    int order[3] = {o0, o1, o2};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i + 1; j < 3; ++j)
            if (d[order[j]] > d[order[i]]) {
                int t = order[i];
                order[i] = order[j];
                order[j] = t;
            }
    double qs[9];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        w[c] = d[order[c]];
#pragma unroll
        for (int r = 0; r < 3; ++r) qs[r * 3 + c] = q[r * 3 + order[c]];
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) q[i] = qs[i];
}

// matrixSquareRoot (tensor.cpp:452-475): L S^(1/2) RT with L = Q, RT = Q^T.
__device__ inline void sqrtm3(const double* A, double* R)
{
    double w[3], q[9], L[9], RT[9], S[9], tmp[9];
    sym3_eig(A, w, q);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            L[i * 3 + j] = q[i * 3 + j];
            RT[i * 3 + j] = q[j * 3 + i];
            S[i * 3 + j] = sqrt(w[i]) * (double)(i == j);
        }
    mm3(L, S, tmp);
    mm3(tmp, RT, R);
}

// ---------------------------------------------------------------------------
// BoxAccessCellArray per-cell operations (boxaccesscellarray.cpp).
// ---------------------------------------------------------------------------
__device__ inline double eff_invG(const DevParams& P, const CellS& c)  // :218-228
{
    double tot = 0.0;
    for (int m = 0; m < P.M; ++m) tot += eos_invG(P, m, ecell_of(c, m));
    return tot;
}
__device__ inline double eff_e_nonthermal(const DevParams& P, const CellS& c)  // :230-240
{
    double tot = 0.0;
    for (int m = 0; m < P.M; ++m) {
        ECell e = ecell_of(c, m);
        tot += (eos_e_cold(P, m, e) + eos_e_shear(P, m, e));
    }
    return tot;
}
__device__ inline double eff_p_nonthermal(const DevParams& P, const CellS& c)  // :242-252
{
    double tot = 0.0;
    for (int m = 0; m < P.M; ++m) {
        ECell e = ecell_of(c, m);
        tot += eos_p_cold(P, m, e) + eos_p_shear(P, m, e);
    }
    return tot;
}

// getDeviatoricHenckyStrain + getHenckyJ2 (:326-380); solids only.
__device__ inline void hencky(const DevParams& P, CellS& c)
{
    if (!P.any_solid) return;
    double B[9], Binv[9], prod[9];
    mmT3(c.V, c.V, B);
    invert3(B, Binv);
#pragma unroll
    for (int q = 0; q < 9; ++q) c.devH[q] = 0.5 * 0.5 * (B[q] - Binv[q]);
    mmT3(c.devH, c.devH, prod);
    c.hj2 = trace3(prod);
}

// stressTensor (:176-216)
__device__ inline void stress(const DevParams& P, CellS& c)
{
    double Gt = 0.0;
    int solid = 0;
    for (int m = 0; m < P.M; ++m)
        if (P.phase[m] == TJ_PHASE_SOLID) {
            ECell e = ecell_of(c, m);
            solid = 1;
            Gt += eos_G(P, m, e) * (eos_invG(P, m, e));
        }
    Gt = Gt / eff_invG(P, c);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            double dl = (double)(r == q);
            c.sigma[3 * r + q] = solid ? (-c.p * dl + 2.0 * Gt * c.devH[3 * r + q]) : (-c.p * dl);
        }
}

// conservativeToPrimitive (:67-122)
__device__ inline void c2p(const DevParams& P, CellS& c)
{
    c.rho = 0;
    for (int m = 0; m < P.M; ++m) {
        c.rhok[m] = c.arho[m] / c.alpha[m];
        c.rho += c.arho[m];
        if (P.plastic && P.phase[m] == TJ_PHASE_SOLID) c.eps[m] = c.are[m] / c.arho[m];
    }
    hencky(P, c);
    double ke = 0.0;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        c.vel[r] = c.rhou[r] / c.rho;
        ke += 0.5 * c.rho * c.vel[r] * c.vel[r];
    }
    c.p = (c.E - ke - eff_e_nonthermal(P, c) + eff_p_nonthermal(P, c)) / (eff_invG(P, c));
    stress(P, c);
}

// primitiveToConservative (:124-174)
__device__ inline void p2c(const DevParams& P, CellS& c)
{
    c.rho = 0;
    for (int m = 0; m < P.M; ++m) {
        c.arho[m] = c.alpha[m] * c.rhok[m];
        c.rho += c.arho[m];
        if (P.plastic && P.phase[m] == TJ_PHASE_SOLID) c.are[m] = c.eps[m] * c.arho[m];
    }
    hencky(P, c);
    double ke = 0.0;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        c.rhou[r] = c.vel[r] * c.rho;
        ke += 0.5 * c.rho * c.vel[r] * c.vel[r];
    }
    c.E = c.p * eff_invG(P, c) + eff_e_nonthermal(P, c) - eff_p_nonthermal(P, c) + ke;
    stress(P, c);
}

// getSoundSpeed (:254-285)
__device__ inline double sound_speed(const DevParams& P, const CellS& c)
{
    double a = 0.0, xit = 0.0;
    for (int m = 0; m < P.M; ++m) {
        ECell e = ecell_of(c, m);
        double xi = 1.0 / gam(P, m);
        double v = xi * eos_c2(P, m, e) * c.arho[m] / c.rho;
        a += (0.0 < v) ? v : 0.0;
        xit += xi * c.alpha[m];
    }
    if (a <= 0.0) a = 1E-6;
    return sqrt(a / xit);
}

// cleanUpAlpha on one cell (:530-599). Returns TJ_ERR_ALPHA on the
// reference's fatal conditions.
__device__ inline int cleanup_alpha(const DevParams& P, double* alpha)
{
    double tot = 0.0;
    int nan = 0;
    for (int m = 0; m < P.M; ++m) {
        double a = alpha[m];
        if (isnan(a)) {
            a = 0.0;
            if (nan == 0) nan = m;
            else return TJ_ERR_ALPHA;
        } else if (a < 0.0) a = 1E-6;
        else if (a > 1.0) a = 1.0;
        alpha[m] = a;
        tot += a;
    }
    if (nan > 0) {
        alpha[nan] = 1.0 - tot;
        tot += alpha[nan];
    }
    if (tot <= 0.0) return TJ_ERR_ALPHA;
    for (int m = 0; m < P.M; ++m) alpha[m] *= 1.0 / tot;
    return 0;
}

// transverseWaveSpeed on a star state (:287-324).
__device__ inline double transverse_speed(const DevParams& P, CellS& c)
{
    hencky(P, c);
    double b = 0.0;
    for (int m = 0; m < P.M; ++m)
        if (P.phase[m] == TJ_PHASE_SOLID) {
            ECell e = ecell_of(c, m);
            b += eos_invG(P, m, e) * eos_G(P, m, e) / (c.rhok[m]);
        }
    if (isnan(b) || b < 0.0) b = 0.0;
    double t = sqrt(b / eff_invG(P, c));
    if (isnan(t)) t = 0.0;
    return t;
}

}  // namespace tj
