// Tangent-linear run of the FP64 update (tj_tangent.cu).
#pragma once

#include <cuda_runtime.h>

#include "tj_fp64.cuh"

namespace tj {

struct TanState;
TanState* tan_create();
void tan_destroy(TanState* t);
// From the primitives prim of domain dom (device, the tj_set_primitive
// layout) with directions dprim (device, NULL: zero) and EOS-parameter
// directions deos (host, [M][TJ_MAX_EOS_PARAMS], NULL: zero), nsteps steps
// with dt[n] (host). Writes the final values (ap, device, may be NULL) and
// directions (dap, device) of the domain in the AccessPattern layout.
// Returns the number of launches, or a negative TJ_ERR_* code.
long long tan_run(TanState* t, const DevParams& P, const Fp64Bufs& b, int dom, const double* prim,
                  const double* dprim, const double* deos, int nsteps, const double* dt, double* ap, double* dap,
                  cudaStream_t st);
int tan_status(TanState* t, int* status, cudaStream_t st);

}  // namespace tj
