// Adjoint (reverse-mode) of the FP64 per-timestep update of one 2-D fluid
// domain with a given time-step schedule.
#pragma once

#include <vector>

#include "tj_fp64.cuh"
#include "tj_types.h"

namespace tj {

struct AdjState;

// Whether the adjoint covers this configuration (2-D, fluids with the
// stiffened-gas Mie-Gruneisen EOS, one domain); the reason otherwise.
const char* adj_unsupported(const DevParams& P, int ndom);

AdjState* adj_create();
void adj_destroy(AdjState* a);

// Runs nsteps steps of dt[n] from the state in b.A (set from the primitives by
// the caller, THINC scratch zeroed), saving the state and the THINC scratch
// every `stride` steps. On return b.A holds the final state. Returns the
// number of kernel launches, or a negative status.
long long adj_forward(AdjState* a, const DevParams& P, const Fp64Bufs& b, const DevDomain& D, const double* dt,
                      int nsteps, int stride, cudaStream_t st);

// From lam_final (device, carried-state layout: the adjoint of the final
// state) to the adjoint of the initial primitives (device, the layout of
// tj_set_primitive) and of the EOS parameters (host, [M][TJ_MAX_EOS_PARAMS]).
// Recomputes each checkpoint interval forward before reversing it. Returns
// the number of kernel launches, or a negative status.
long long adj_backward(AdjState* a, const DevParams& P, const Fp64Bufs& b, const DevDomain& D, const double* lam_final,
                       double* grad_prim, double* grad_eos, cudaStream_t st);

// Bytes of device memory the adjoint holds.
size_t adj_bytes(const AdjState* a);

}  // namespace tj
