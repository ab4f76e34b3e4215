/* Interposes the pinned transcendental functions of tj_libm.h over libm's
 * symbols in the oracle's reference binaries (test infrastructure only). */
#include "tj_libm.h"

double exp(double x) { return tjm_exp(x); }
double log(double x) { return tjm_log(x); }
double pow(double x, double y) { return tjm_pow(x, y); }
double cosh(double x) { return tjm_cosh(x); }
double tanh(double x) { return tjm_tanh(x); }
