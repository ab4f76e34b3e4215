// Mixed-precision path: not yet built; contexts asking for it are refused.
#include "tj_mixed.cuh"

namespace tj {

bool mixed_supported(const tj_params&) { return false; }
int mixed_alloc(MixedState&, const DevParams&, const std::vector<DevDomain>&, long long, const long long*, cudaStream_t) { return TJ_ERR_ARG; }
void mixed_free(MixedState&) {}
int mixed_set_boxes(MixedState&, const DevParams&, const std::vector<DevDomain>&, const std::vector<std::vector<int>>&, cudaStream_t) { return TJ_OK; }
int mixed_from_fp64(MixedState&, const DevParams&, const Fp64Bufs&, cudaStream_t) { return 0; }
int mixed_to_fp64(MixedState&, const DevParams&, const Fp64Bufs&, cudaStream_t) { return 0; }
int mixed_compute_dt(MixedState&, const DevParams&, const Fp64Bufs&, cudaStream_t) { return 0; }
int mixed_step(MixedState&, const DevParams&, const Fp64Bufs&, cudaStream_t, Prof*) { return 0; }
int mixed_launches_per_step(const DevParams&) { return 0; }

}  // namespace tj
