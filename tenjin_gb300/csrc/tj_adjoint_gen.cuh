// Reverse mode of the FP64 update for every configuration but BVD-THINC and
// mixtures, by local Jacobians of the Dual instance (tj_adjoint_gen.cu).
#pragma once

#include <cuda_runtime.h>

#include "tj_fp64.cuh"

namespace tj {

struct GenAdj;
GenAdj* gen_create();
void gen_destroy(GenAdj* a);
// NULL when the general reverse mode covers the configuration, else why not.
const char* gen_unsupported(const DevParams& P, int ndom);
// nsteps FP64 steps of b.A (already the initial state of the primitives prim,
// device, nprim words per cell) with dt[n] (host), checkpointing b.A every
// `stride` steps. Returns the number of launches or a negative TJ_ERR_*.
long long gen_forward(GenAdj* a, const DevParams& P, const Fp64Bufs& b, const double* prim, int nprim, const double* dt,
                      int nsteps, int stride, cudaStream_t st);
// From grad_ap (device, AccessPattern layout of the domain) to grad_prim
// (device, the primitives' layout) and grad_eos (host,
// [M][TJ_MAX_EOS_PARAMS]); nparams[m]: parameters of material m.
long long gen_backward(GenAdj* a, const DevParams& P, const Fp64Bufs& b, const double* grad_ap, double* grad_prim,
                       double* grad_eos, const int* nparams, cudaStream_t st);

}  // namespace tj
