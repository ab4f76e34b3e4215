// Launchers of the per-direction kernels (tj_path.cuh) for one working type.
// Each (material count, direction) pair with M = 1 or 2 has its own instance,
// in which both are compile-time constants: the per-material loops unroll,
// the cell structures stay in registers and every direction-indexed access
// is static. M = 3 and 4 use the generic instance (runtime M and direction).
// The instances are compiled in separate translation units
// (tj_path_inst.cu, once per type, M and direction) so that they build in
// parallel.
#pragma once

#include <cuda_runtime.h>

#include "tj_fp64.cuh"

namespace tj {

// One direction of one RK stage: k_recon, k_flux, k_update. Returns the
// number of launches.
template <class PT, int DC>
int path_dir(const PT& P, const PathBufs<typename PT::real>& b, const typename PT::real* X, typename PT::real* Y,
             int d, int first, int last, int finish, cudaStream_t st, Prof* pr);
// The CFL pass (k_cfl) over the state X.
template <class PT>
int path_cfl(const PT& P, const PathBufs<typename PT::real>& b, const typename PT::real* X, cudaStream_t st,
             Prof* pr);

template <class Base>
inline int path_dir_any(const Base& P, const PathBufs<typename Base::real>& b, const typename Base::real* X,
                        typename Base::real* Y, int d, int first, int last, int finish, cudaStream_t st, Prof* pr)
{
    switch (P.M * 4 + d) {
        case 4: return path_dir<WithM<Base, 1>, 0>(WithM<Base, 1>(P), b, X, Y, d, first, last, finish, st, pr);
        case 5: return path_dir<WithM<Base, 1>, 1>(WithM<Base, 1>(P), b, X, Y, d, first, last, finish, st, pr);
        case 6: return path_dir<WithM<Base, 1>, 2>(WithM<Base, 1>(P), b, X, Y, d, first, last, finish, st, pr);
        case 8: return path_dir<WithM<Base, 2>, 0>(WithM<Base, 2>(P), b, X, Y, d, first, last, finish, st, pr);
        case 9: return path_dir<WithM<Base, 2>, 1>(WithM<Base, 2>(P), b, X, Y, d, first, last, finish, st, pr);
        case 10: return path_dir<WithM<Base, 2>, 2>(WithM<Base, 2>(P), b, X, Y, d, first, last, finish, st, pr);
        default: return path_dir<Base, -1>(P, b, X, Y, d, first, last, finish, st, pr);
    }
}

template <class Base>
inline int path_cfl_any(const Base& P, const PathBufs<typename Base::real>& b, const typename Base::real* X,
                        cudaStream_t st, Prof* pr)
{
    if (P.M == 1) return path_cfl<WithM<Base, 1>>(WithM<Base, 1>(P), b, X, st, pr);
    if (P.M == 2) return path_cfl<WithM<Base, 2>>(WithM<Base, 2>(P), b, X, st, pr);
    return path_cfl<Base>(P, b, X, st, pr);
}

}  // namespace tj
