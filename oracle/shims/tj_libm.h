/* Pinned transcendental functions for the oracle (test infrastructure only).
 *
 * The reference calls exp, cosh, tanh (thinc.cpp:131-134), pow
 * (equationofstate.cpp:421-449, boxaccesscellarray.cpp:514) and log
 * (equationofstate.cpp:523) from whatever libm it is linked with; their last
 * bit differs between libm builds (and differs from the GPU's), and a
 * one-ulp difference inside BVD-THINC can flip a limiter branch a few steps
 * later. The oracle therefore pins libm: these definitions are linked into the
 * reference binaries (interposing the libm symbols) and used by the port, and
 * the GPU code restates the same algorithms. Every function uses only IEEE
 * +,-,*,/ (no contraction), floor, frexp and ldexp, so it gives the same bits
 * on any IEEE machine.
 *   exp:  Cody-Waite reduction x = k ln2 + r, |r| <= ln2/2, ln2 split into a
 *         32-bit head and a tail; e^r by its Taylor series to degree 13 in
 *         Horner form; scaled by 2^k.
 *   log:  x = 2^e m with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
 *         s = (m-1)/(m+1), series in s^2 to degree 12.
 *   pow:  exp(y log x) for x > 0.
 *   expm1: the same Taylor series without its constant term for |x| <= 0.35,
 *         exp(x) - 1 otherwise.
 *   cosh: (e^|x| + e^-|x|)/2;  tanh: t/(t+2) with t = expm1(2|x|), sign of x.
 * Accuracy is about one ulp over the ranges the path uses.
 */
#ifndef TJ_ORACLE_LIBM_H
#define TJ_ORACLE_LIBM_H

#include <math.h>

#define TJM_LN2_HI 0x1.62e42fee00000p-1 /* ln 2 to 32 significant bits */
#define TJM_LN2_LO 0x1.a39ef35793c76p-33 /* ln 2 - TJM_LN2_HI */
#define TJM_INV_LN2 0x1.71547652b82fep+0
#define TJM_SQRT_HALF 0x1.6a09e667f3bcdp-1

static inline double tjm_exp(double x)
{
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    double kd = x * TJM_INV_LN2;
    kd = (kd >= 0.0) ? floor(kd + 0.5) : -floor(-kd + 0.5);
    double r = (x - kd * TJM_LN2_HI) - kd * TJM_LN2_LO;
    /* 1/n! rounded to nearest, n = 13 .. 0 */
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
    p = p * r + 1.0;
    return ldexp(p, (int)kd);
}

static inline double tjm_expm1(double x)
{
    if (x != x) return x;
    if (fabs(x) > 0.35) return tjm_exp(x) - 1.0;
    double p = 0x1.6124613a86d09p-33;
    p = p * x + 0x1.1eed8eff8d898p-29;
    p = p * x + 0x1.ae64567f544e4p-26;
    p = p * x + 0x1.27e4fb7789f5cp-22;
    p = p * x + 0x1.71de3a556c734p-19;
    p = p * x + 0x1.a01a01a01a01ap-16;
    p = p * x + 0x1.a01a01a01a01ap-13;
    p = p * x + 0x1.6c16c16c16c17p-10;
    p = p * x + 0x1.1111111111111p-7;
    p = p * x + 0x1.5555555555555p-5;
    p = p * x + 0x1.5555555555555p-3;
    p = p * x + 0x1.0000000000000p-1;
    p = p * x + 1.0;
    return p * x;
}

static inline double tjm_log(double x)
{
    if (x != x) return x;
    if (x < 0.0) return NAN;
    if (x == 0.0) return -INFINITY;
    if (x == INFINITY) return x;
    int e;
    double m = frexp(x, &e);
    if (m < TJM_SQRT_HALF) { m = m * 2.0; e = e - 1; }
    double f = m - 1.0;
    double s = f / (2.0 + f);
    double z = s * s;
    /* 1/(2k+1), k = 12 .. 0 */
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

static inline double tjm_pow(double x, double y)
{
    if (y == 0.0 || x == 1.0) return 1.0;
    if (x != x || y != y) return x + y;
    if (x == 0.0) return (y > 0.0) ? 0.0 : INFINITY;
    if (x < 0.0) return NAN;
    if (x == INFINITY) return (y > 0.0) ? INFINITY : 0.0;
    return tjm_exp(y * tjm_log(x));
}

static inline double tjm_cosh(double x)
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

static inline double tjm_tanh(double x)
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

#endif
