// Transcendental functions of the FP64 reference-faithful path.
//
// The reference takes exp, cosh, tanh, pow and log from the host libm, whose
// last bit is not specified; a one-ulp difference inside BVD-THINC can flip a
// limiter branch steps later. The FP64 path therefore uses its own
// deterministic implementations, built only from IEEE +,-,*,/ (compiled with
// -fmad=false), floor, frexp and ldexp, so the same arguments give the same
// bits on the GPU and on any IEEE host; the parity oracle is pinned to the
// same algorithms.
//   exp:   Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2 (ln2 split into a
//          32-bit head and a tail), Taylor series of e^r to degree 13 in Horner
//          form, scaled by 2^k.
//   expm1: the same series without its constant term for |x| <= 0.35.
//   log:   x = 2^e m, m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
//          s = (m-1)/(m+1), series in s^2 to degree 12.
//   pow:   exp(y log x), x > 0.   cosh: (e^|x| + e^-|x|)/2.
//   tanh:  t/(t+2), t = expm1(2|x|), with the sign of x.
#pragma once

namespace tj {

#define TJM_LN2_HI 0x1.62e42fee00000p-1
#define TJM_LN2_LO 0x1.a39ef35793c76p-33
#define TJM_INV_LN2 0x1.71547652b82fep+0
#define TJM_SQRT_HALF 0x1.6a09e667f3bcdp-1

// Taylor coefficients 1/n!, n = 13 .. 2, rounded to nearest.
__device__ __forceinline__ double tjm_exp_series(double r)
{
    double p = 0x1.6124613a86d09p-33;
    p = p * r + 0x1.1eed8eff8d898p-29;
    p = p * r + 0x1.ae64567f544e4p-26;
    p = p * r + 0x1.27e4fb7789f5cp-22;
    p = p * r + 0x1.71de3a556c734p-19;
    p = p * r + 0x1.a01a01a01a01ap-16;
    p = p * r + 0x1.a01a01a01a01ap-13;
    p = p * r + 0x1.6c16c16c16c17p-10;
    p = p * r + 0x1.1111111111111p-7;
    p = p * r + 0x1.5555555555555p-5;
    p = p * r + 0x1.5555555555555p-3;
    p = p * r + 0x1.0000000000000p-1;
    p = p * r + 1.0;
    return p;  // (e^r - 1)/r
}

__device__ inline double tjm_exp(double x)
{
    if (x != x) return x;
    if (x > 709.782712893384) return __longlong_as_double(0x7ff0000000000000ll);
    if (x < -745.1332191019412) return 0.0;
    double kd = x * TJM_INV_LN2;
    kd = (kd >= 0.0) ? floor(kd + 0.5) : -floor(-kd + 0.5);
    double r = (x - kd * TJM_LN2_HI) - kd * TJM_LN2_LO;
    double p = tjm_exp_series(r);
    p = p * r + 1.0;
    return ldexp(p, (int)kd);
}

__device__ inline double tjm_expm1(double x)
{
    if (x != x) return x;
    if (fabs(x) > 0.35) return tjm_exp(x) - 1.0;
    return tjm_exp_series(x) * x;
}

__device__ inline double tjm_log(double x)
{
    if (x != x) return x;
    if (x < 0.0) return __longlong_as_double(0x7ff8000000000000ll);
    if (x == 0.0) return -__longlong_as_double(0x7ff0000000000000ll);
    if (isinf(x)) return x;
    int e;
    double m = frexp(x, &e);
    if (m < TJM_SQRT_HALF) {
        m = m * 2.0;
        e = e - 1;
    }
    double f = m - 1.0;
    double s = f / (2.0 + f);
    double z = s * s;
    // 1/(2k+1), k = 12 .. 0, rounded to nearest
    double q = 0x1.47ae147ae147bp-5;
    q = q * z + 0x1.642c8590b2164p-5;
    q = q * z + 0x1.8618618618618p-5;
    q = q * z + 0x1.af286bca1af28p-5;
    q = q * z + 0x1.e1e1e1e1e1e1ep-5;
    q = q * z + 0x1.1111111111111p-4;
    q = q * z + 0x1.3b13b13b13b14p-4;
    q = q * z + 0x1.745d1745d1746p-4;
    q = q * z + 0x1.c71c71c71c71cp-4;
    q = q * z + 0x1.2492492492492p-3;
    q = q * z + 0x1.999999999999ap-3;
    q = q * z + 0x1.5555555555555p-2;
    q = q * z + 1.0;
    double lm = (2.0 * s) * q;
    double ed = (double)e;
    return ed * TJM_LN2_HI + (lm + ed * TJM_LN2_LO);
}

__device__ inline double tjm_pow(double x, double y)
{
    if (y == 0.0 || x == 1.0) return 1.0;
    if (x != x || y != y) return x + y;
    if (x == 0.0) return (y > 0.0) ? 0.0 : __longlong_as_double(0x7ff0000000000000ll);
    if (x < 0.0) return __longlong_as_double(0x7ff8000000000000ll);
    if (isinf(x)) return (y > 0.0) ? x : 0.0;
    return tjm_exp(y * tjm_log(x));
}

__device__ inline double tjm_cosh(double x)
{
    double a = fabs(x);
    if (a != a) return a;
    if (a > 709.0) {
        double t = tjm_exp(0.5 * a);
        return (0.5 * t) * t;
    }
    double t = tjm_exp(a);
    return 0.5 * t + 0.5 / t;
}

__device__ inline double tjm_tanh(double x)
{
    double a = fabs(x);
    if (a != a) return x;
    double r;
    if (a > 22.0) r = 1.0;
    else {
        double t = tjm_expm1(2.0 * a);
        r = t / (t + 2.0);
    }
    return copysign(r, x);
}

// binary32 overloads (the binary32 instance of the kernels; fast-math library calls)
__device__ inline float tjm_exp(float x) { return expf(x); }
__device__ inline float tjm_expm1(float x) { return expm1f(x); }
__device__ inline float tjm_log(float x) { return logf(x); }
__device__ inline float tjm_pow(float x, float y) { return powf(x, y); }
__device__ inline float tjm_cosh(float x) { return coshf(x); }
__device__ inline float tjm_tanh(float x) { return tanhf(x); }

}  // namespace tj
