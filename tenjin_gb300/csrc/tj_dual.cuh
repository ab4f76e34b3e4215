// Forward-mode (tangent-linear) arithmetic for the per-direction kernels:
// a binary64 value and one binary64 directional derivative. The value part
// of every operation is the binary64 operation the FP64 instance performs
// (the unit is compiled without contraction, like that instance), so a
// tangent run takes the FP64 path's branches and reproduces its values bit
// for bit; the derivative part is the chain rule of that operation. Branches
// (limiter, clamps, Riemann-solver sides, the radial return's yield test) are
// differentiated at their taken side.
#pragma once

#include <cuda_runtime.h>

#include "tj_device.cuh"
#include "tj_math.cuh"
#include "tj_types.h"

namespace tj {

struct Dual {
    double v, d;
    Dual() = default;
    __host__ __device__ constexpr Dual(double x) : v(x), d(0.0) {}
    __host__ __device__ constexpr Dual(double x, double t) : v(x), d(t) {}
};

// A zero direction contributes nothing, whatever the partial derivative is
// (an infinite or undefined quotient the value side discards, such as the
// limiter ratio of a uniform state): every product with a direction is
// taken only when that direction is nonzero.
__device__ __forceinline__ double dmul(double t, double x) { return t != 0.0 ? t * x : 0.0; }

__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, dmul(a.d, b.v) + dmul(b.d, a.v)); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b)
{
    const double q = a.v / b.v;
    return Dual(q, (b.d != 0.0 ? (a.d - q * b.d) / b.v : (a.d != 0.0 ? a.d / b.v : 0.0)));
}
__device__ __forceinline__ Dual operator+(Dual a, double b) { return Dual(a.v + b, a.d); }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return Dual(a + b.v, b.d); }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return Dual(a.v - b, a.d); }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return Dual(a - b.v, -b.d); }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return Dual(a.v * b, dmul(a.d, b)); }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return Dual(a * b.v, dmul(b.d, a)); }
__device__ __forceinline__ Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d != 0.0 ? a.d / b : 0.0); }
__device__ __forceinline__ Dual operator/(double a, Dual b)
{
    const double q = a / b.v;
    return Dual(q, b.d != 0.0 ? -q * b.d / b.v : 0.0);
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { return a = a + b; }
__device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) { return a = a - b; }
__device__ __forceinline__ Dual& operator*=(Dual& a, Dual b) { return a = a * b; }
__device__ __forceinline__ Dual& operator/=(Dual& a, Dual b) { return a = a / b; }

#define TJ_DUAL_CMP(op)                                                                        \
    __device__ __forceinline__ bool operator op(Dual a, Dual b) { return a.v op b.v; }     \
    __device__ __forceinline__ bool operator op(Dual a, double b) { return a.v op b; }     \
    __device__ __forceinline__ bool operator op(double a, Dual b) { return a op b.v; }
TJ_DUAL_CMP(<)
TJ_DUAL_CMP(>)
TJ_DUAL_CMP(<=)
TJ_DUAL_CMP(>=)
TJ_DUAL_CMP(==)
TJ_DUAL_CMP(!=)
#undef TJ_DUAL_CMP

// the binary64 / binary32 overloads stay visible next to the Dual ones
using ::fabs;
using ::isinf;
using ::isnan;
using ::sqrt;

__device__ __forceinline__ bool isnan(Dual a) { return ::isnan(a.v); }
__device__ __forceinline__ bool isinf(Dual a) { return ::isinf(a.v); }
__device__ __forceinline__ Dual fabs(Dual a) { return a.v < 0.0 ? -a : a; }
// d sqrt(x) = dx / (2 sqrt(x)); a zero direction stays zero at x = 0 (the
// Hencky J2 of an undeformed cell)
__device__ __forceinline__ Dual sqrt(Dual a)
{
    const double s = ::sqrt(a.v);
    return Dual(s, a.d == 0.0 ? 0.0 : a.d / (2.0 * s));
}
__device__ __forceinline__ Dual tjm_exp(Dual a)
{
    const double e = tjm_exp(a.v);
    return Dual(e, dmul(a.d, e));
}
__device__ __forceinline__ Dual tjm_log(Dual a) { return Dual(tjm_log(a.v), a.d != 0.0 ? a.d / a.v : 0.0); }
__device__ __forceinline__ Dual tjm_pow(Dual x, Dual y)
{
    const double p = tjm_pow(x.v, y.v);
    double d = 0.0;
    if (x.d != 0.0) d += p * y.v * x.d / x.v;
    if (y.d != 0.0) d += p * ::log(x.v) * y.d;
    return Dual(p, d);
}
__device__ __forceinline__ Dual tjm_cosh(Dual a) { return Dual(tjm_cosh(a.v), dmul(a.d, ::sinh(a.v))); }
__device__ __forceinline__ Dual tjm_tanh(Dual a)
{
    const double t = tjm_tanh(a.v);
    return Dual(t, dmul(a.d, 1.0 - t * t));
}

// Equality of the values' bit patterns (the repeated cleanUpAlpha's
// convergence test).
__device__ __forceinline__ bool same_bits(Dual a, Dual b)
{
    return __double_as_longlong(a.v) == __double_as_longlong(b.v);
}

// matrixSquareRoot (tensor.cpp:452-475) with a direction: the values by the
// binary64 routine itself; the direction solves the Sylvester equation
// S dS + dS S = dA in A's eigenbasis, dS'_ij = dA'_ij / (sqrt(w_i) + sqrt(w_j)),
// which is exact also where eigenvalues repeat (the undeformed V = I), where
// differentiating the Jacobi rotations is not.
__device__ inline void sqrtm3(const Dual* A, Dual* Rm)
{
    double a[9], da[9], r[9], w[3], q[9];
    bool any = false;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        a[i] = A[i].v;
        da[i] = A[i].d;
        any |= da[i] != 0.0;
    }
    sqrtm3(a, r);
    if (!any) {
#pragma unroll
        for (int i = 0; i < 9; ++i) Rm[i] = Dual(r[i]);
        return;
    }
    sym3_eig(a, w, q);
    double t[9], dp[9], ds[9];
    // dA' = Q^T dA Q
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = da[i * 3 + 0] * q[0 * 3 + j] + da[i * 3 + 1] * q[1 * 3 + j] + da[i * 3 + 2] * q[2 * 3 + j];
    double sw[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) sw[i] = ::sqrt(w[i] > 0.0 ? w[i] : 0.0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double v = q[0 * 3 + i] * t[0 * 3 + j] + q[1 * 3 + i] * t[1 * 3 + j] + q[2 * 3 + i] * t[2 * 3 + j];
            const double den = sw[i] + sw[j];
            dp[i * 3 + j] = den > 0.0 ? v / den : 0.0;
        }
    // dS = Q dS' Q^T
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = q[i * 3 + 0] * dp[0 * 3 + j] + q[i * 3 + 1] * dp[1 * 3 + j] + q[i * 3 + 2] * dp[2 * 3 + j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) ds[i * 3 + j] = t[i * 3 + 0] * q[j * 3 + 0] + t[i * 3 + 1] * q[j * 3 + 1] + t[i * 3 + 2] * q[j * 3 + 2];
#pragma unroll
    for (int i = 0; i < 9; ++i) Rm[i] = Dual(r[i], ds[i]);
}

// The parameter block of the tangent instance: the FP64 layout with the
// EOS parameters (and the yield stresses) as values with directions, so that
// derivatives along the EOS parameters come out of the same run.
struct DevParamsT {
    using real = Dual;
    int dim, M, solid, thinc, plastic, muscl, any_solid;
    int fused64;
    int radial;
    int nmix, reactive;
    int lo_bc[3], hi_bc[3];
    Dual cfl, beta;
    int phase[TJ_MAX_MAT], eos[TJ_MAX_MAT];
    Dual prm[TJ_MAX_MAT][TJ_MAX_EOS_PARAMS];
    Dual yield[TJ_MAX_MAT];
    int S_ALPHA, S_ARHO, S_RHOK, S_RHO, S_RHOU, S_VEL, S_E, S_P, S_V, S_HJ2, S_EPS, S_ARE, NS;
    int S_RMIX, S_LAM, S_ARL;
    int F_ALPHA, F_ARHO, F_RHO, F_RHOU, F_VEL, F_E, F_P, F_A, F_SIGMA, F_V, F_ARE, NF;
    int F_ARL;
    int X_ALPHA, X_ARHO, X_RHOU, X_E, X_SSTAR, X_V, X_VSTAR, X_ARE, NX;
    int X_ARL;
    int S_ELO;
};

}  // namespace tj
