/* Test harness (not part of the library): the oracle's host build of the
 * same transcendental algorithms (oracle/shims/tj_libm.h), compiled with the
 * oracle's flags, evaluated over an array. */
#include "tj_libm.h"

void tjm_eval_host(int fn, const double* x, const double* y, int n, double* out)
{
    for (int i = 0; i < n; ++i) {
        switch (fn) {
            case 0: out[i] = tjm_exp(x[i]); break;
            case 1: out[i] = tjm_log(x[i]); break;
            case 2: out[i] = tjm_pow(x[i], y[i]); break;
            case 3: out[i] = tjm_cosh(x[i]); break;
            case 4: out[i] = tjm_tanh(x[i]); break;
            case 5: out[i] = tjm_expm1(x[i]); break;
            default: out[i] = 0.0;
        }
    }
}
