// One instance of the per-direction launchers (tj_path_launch.cuh), selected
// at compile time: TJ_INST_R = 64 (binary64, DevParams) or 32 (binary32,
// DevParams32); TJ_INST_M = material count, 0 for the generic instance;
// TJ_INST_D = direction, -1 for the generic instance; TJ_INST_R = 128 is the
// tangent instance (DevParamsT, tj_dual.cuh), which has no CFL pass. The CFL
// pass is instantiated with the first direction of each material count.
#if defined(TJ_INST_R) && TJ_INST_R == 128
#include "tj_dual.cuh"
#endif
#include "tj_path.cuh"
#include "tj_path_launch.cuh"
#if defined(TJ_INST_R) && TJ_INST_R == 128
#include "tj_dual_path.cuh"
#endif

#if !defined(TJ_INST_R) || !defined(TJ_INST_M) || !defined(TJ_INST_D)
#error "TJ_INST_R, TJ_INST_M and TJ_INST_D select the instance"
#endif

namespace tj {

namespace {
constexpr int kPathThreads = 256;
inline int path_blocks(long long n, int cap = 152 * 16)
{
    long long b = (n + kPathThreads - 1) / kPathThreads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}
}  // namespace

template <class PT, int DC>
int path_dir(const PT& P, const PathBufs<typename PT::real>& b, const typename PT::real* X, typename PT::real* Y,
             int d, int first, int last, int finish, cudaStream_t st, Prof* pr)
{
    constexpr bool f64 = sizeof(typename PT::real) == 8;
    const char* nr = f64 ? "tj_recon_fp64" : "tj_recon_fp32";
    const char* nf = f64 ? "tj_flux_fp64" : "tj_flux_fp32";
    const char* nu = f64 ? "tj_update_fp64" : "tj_update_fp32";
    if (pr) pr->begin(nr, st);
    k_recon<PT, DC><<<path_blocks(b.ntot), kPathThreads, 0, st>>>(P, b, X, d);
    if (pr) pr->end(nr, st);
    if (pr) pr->begin(nf, st);
    k_flux<PT, DC><<<path_blocks(b.nftot[d]), kPathThreads, 0, st>>>(P, b, d);
    if (pr) pr->end(nf, st);
    if (pr) pr->begin(nu, st);
    k_update<PT, DC><<<path_blocks(b.ntot), kPathThreads, 0, st>>>(P, b, X, Y, d, first, last, finish);
    if (pr) pr->end(nu, st);
    return 3;
}

template <class PT>
int path_cfl(const PT& P, const PathBufs<typename PT::real>& b, const typename PT::real* X, cudaStream_t st, Prof* pr)
{
    const char* nc = sizeof(typename PT::real) == 8 ? "tj_cfl_fp64" : "tj_cfl_fp32";
    if (pr) pr->begin(nc, st);
    k_cfl<<<path_blocks(b.ntot), kPathThreads, 0, st>>>(P, b, X);
    if (pr) pr->end(nc, st);
    return 1;
}

#if TJ_INST_R == 64
using InstBase = DevParams;
#elif TJ_INST_R == 128
using InstBase = DevParamsT;
#else
using InstBase = DevParams32;
#endif
#if TJ_INST_M > 0
using InstPT = WithM<InstBase, TJ_INST_M>;
#else
using InstPT = InstBase;
#endif

template int path_dir<InstPT, TJ_INST_D>(const InstPT&, const PathBufs<InstPT::real>&, const InstPT::real*,
                                         InstPT::real*, int, int, int, int, cudaStream_t, Prof*);
#if TJ_INST_D <= 0 && TJ_INST_R != 128
template int path_cfl<InstPT>(const InstPT&, const PathBufs<InstPT::real>&, const InstPT::real*, cudaStream_t, Prof*);
#endif

}  // namespace tj
