// Fused stage kernels of the per-timestep update: 2-D (binary32 or binary64
// working type) and 3-D over many domains (binary32).
#pragma once

#include <vector>

#include "tj_fp64.cuh"
#include "tj_types.h"

namespace tj {

struct MixedState {
    bool allocated = false;
    void* impl = nullptr;
};

// One fused implementation (2-D single domain; 3-D many domains).
struct MixedBase {
    virtual ~MixedBase() {}
    virtual int set_boxes(const std::vector<DevDomain>& doms, const std::vector<std::vector<int>>& boxes,
                          cudaStream_t st) = 0;
    virtual int from_fp64(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st) = 0;
    virtual int to_fp64(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st) = 0;
    // Whole-domain AccessPattern planes (ngrow 0, possibly a page-locked host
    // buffer read in place) -> both the FP64 carried state and the mixed state,
    // the next step's CFL minimum armed; returns the launches, -1 where the
    // implementation has no such pass. Waits for the stream.
    virtual int from_ap(const DevParams& DP, const Fp64Bufs& fb, const double* ap, cudaStream_t st)
    {
        (void)DP, (void)fb, (void)ap, (void)st;
        return -1;
    }
    virtual int cfl(const Fp64Bufs& fb, cudaStream_t st) = 0;
    virtual int step(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st, Prof* pr) = 0;
    // a one-line description of the launch configuration in use
    virtual void describe(char* buf, size_t len) const
    {
        if (len) buf[0] = 0;
    }
};

// The binary32 per-direction kernels for every other configuration (tj_fp32.cu).
MixedBase* general32_create(const DevParams& DP, long long ntot, const long long* nftot, cudaStream_t st, int* err);

// The 3-D fluid implementation (tj_mixed3d.cu).
MixedBase* mixed3d_create(const DevParams& DP, const std::vector<DevDomain>& doms, long long ntot, cudaStream_t st,
                          int* err);

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
int mixed_from_ap(MixedState& m, const DevParams& P, const Fp64Bufs& b, const double* ap, cudaStream_t st);
// CFL minimum of the current mixed state into DevScalars::dtmin_bits.
int mixed_compute_dt(MixedState& m, const DevParams& P, const Fp64Bufs& b, cudaStream_t st);
int mixed_step(MixedState& m, const DevParams& P, const Fp64Bufs& b, cudaStream_t st, Prof* pr = nullptr);
int mixed_launches_per_step(const DevParams& P);
void mixed_describe(const MixedState& m, char* buf, size_t len);

}  // namespace tj
