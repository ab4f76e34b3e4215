// Overloads of the per-direction kernels' device functions for the tangent
// instance (tj_dual.cuh) that differentiate an expression in a form other
// than the one its value is computed in. Included after tj_path.cuh.
#pragma once

#include "tj_dual.cuh"
#include "tj_path.cuh"

namespace tj {

// MUSCLextrapolate of one variable (hllc.cpp:527-568) with a direction: the
// values by the binary64 expression itself; the direction by the active
// branch. The van Leer slope of this form equals u0 - um where 0 < r < 1,
// up - u0 where r >= 1 and 0 otherwise, so its derivative is that of the
// difference; differentiating through the ratio r instead cancels two large
// terms in nearly uniform regions (where up - u0 is a rounding residue) and
// can leave inf - inf.
__device__ inline void muscl1(Dual um, Dual u0, Dual up, Dual& l, Dual& r)
{
    double lv, rv;
    muscl1(um.v, u0.v, up.v, lv, rv);
    double rr = (u0.v - um.v) / (up.v - u0.v);
    if (isinf(rr) || isnan(rr)) rr = 0.0;
    double dg = 0.0;
    if (rr > 0.0) {
        const double a = 2.0 / (1.0 + rr), b = 2.0 * rr / (1.0 + rr);
        dg = (b < a) ? u0.d - um.d : up.d - u0.d;
    }
    l = Dual(lv, u0.d - 0.5 * dg);
    r = Dual(rv, u0.d + 0.5 * dg);
}

}  // namespace tj
