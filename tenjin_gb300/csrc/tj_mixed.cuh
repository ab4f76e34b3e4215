// Mixed-precision (binary32 bulk) fused kernels of the per-timestep update.
#pragma once

#include <vector>

#include "tj_fp64.cuh"
#include "tj_types.h"

namespace tj {

struct MixedState {
    bool allocated = false;
    void* impl = nullptr;
};

bool mixed_supported(const tj_params& p);
int mixed_alloc(MixedState& m, const DevParams& P, const std::vector<DevDomain>& doms, long long ntot,
                const long long* nftot, cudaStream_t st);
void mixed_free(MixedState& m);
int mixed_set_boxes(MixedState& m, const DevParams& P, const std::vector<DevDomain>& doms,
                    const std::vector<std::vector<int>>& boxes, cudaStream_t st);
// Convert the FP64 carried state (Fp64Bufs::A) into the mixed state and arm
// the next step's CFL minimum; and back.
int mixed_from_fp64(MixedState& m, const DevParams& P, const Fp64Bufs& b, cudaStream_t st);
int mixed_to_fp64(MixedState& m, const DevParams& P, const Fp64Bufs& b, cudaStream_t st);
// CFL minimum of the current mixed state into DevScalars::dtmin_bits.
int mixed_compute_dt(MixedState& m, const DevParams& P, const Fp64Bufs& b, cudaStream_t st);
int mixed_step(MixedState& m, const DevParams& P, const Fp64Bufs& b, cudaStream_t st, Prof* pr = nullptr);
int mixed_launches_per_step(const DevParams& P);

}  // namespace tj
