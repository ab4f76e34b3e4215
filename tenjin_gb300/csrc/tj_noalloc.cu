// CFL time step without any device allocation (tj_compute_dt_noalloc).
//
// Some callers cannot allocate device memory themselves: a host application
// that has handed the whole GPU to a framework's memory pool (which then owns
// every byte it preallocated), a plugin that may only use buffers its host
// gives it, or a time loop that must not pay for, or fail on, an allocation
// once it is running. They can still compute the time step of a state they
// already hold on the GPU with this entry point: the caller passes the state
// (input, device memory) and receives dt (output, host memory); the only
// working memory is the file-scope array below, which is part of the loaded
// library image, so nothing is allocated per call.
//
// The kernels are the CFL reduction of the FP64 path (TimeStep::getTimeStep,
// timestep.cpp:36-70: sound speed by getSoundSpeed, boxaccesscellarray.cpp:
// 254-285, then CFL * min over cells and directions of dx/(a + |u|)) with the
// reduction's accumulator moved from context memory into that array.
//
// The array is shared by every call on a device and keeps the last call's
// partial minima; each call overwrites every slot it reads, so no clearing is
// needed. Calls whose kernels overlap on the GPU (from several host threads,
// or on several streams without ordering) race on the array and may return
// wrong results: serialise them. Every GPU that loads the library holds the
// array (about 64 KiB) until the process exits.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress, with that device current, and caches it. Make
// that first call before any stream capture begins.
//
// Every call copies dt into host memory and synchronises the stream, so no
// call may be made while that stream is being captured into a graph.
//
// The arithmetic is binary64 whatever the precision field of the parameters
// says: dt is the one tj_compute_dt gives for a TJ_PRECISION_FP64 context on
// the same state (a context that carries binary32 state computes its own dt
// from that state, which differs by rounding).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "tj_device.cuh"
#include "tj_layout.h"
#include "tj_types.h"

namespace tj {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaCellsPerBlock = kNaThreads * 8;
constexpr int kNaMaxBlocks = TJ_NOALLOC_MAX_CELLS / kNaCellsPerBlock;

// Partial minima of the blocks of the first pass, then the result.
static __device__ __align__(256) double tj_noalloc_scratch[kNaMaxBlocks + 1];

struct NaLayout {
    int M, dim, solid;
    int A_ALPHA, A_ARHO, A_RHOK, A_RHO, A_VEL, A_P, A_HJ2;
    long long N;
    int n[3];
    double dx[3], cfl;
};

__global__ void k_na_cfl_partial(DevParams P, NaLayout L, const double* __restrict__ st, double* scratch)
{
    double mn = 1.79769313486231570815e+308;
    const long long base = (long long)blockIdx.x * kNaCellsPerBlock;
    for (int k = threadIdx.x; k < kNaCellsPerBlock; k += kNaThreads) {
        const long long g = base + k;
        if (g >= L.N) break;
        CellS c;
        for (int m = 0; m < L.M; ++m) {
            c.alpha[m] = st[(L.A_ALPHA + m) * L.N + g];
            c.arho[m] = st[(L.A_ARHO + m) * L.N + g];
            c.rhok[m] = st[(L.A_RHOK + m) * L.N + g];
        }
        c.rho = st[L.A_RHO * L.N + g];
        c.p = st[L.A_P * L.N + g];
        c.hj2 = L.solid ? st[L.A_HJ2 * L.N + g] : 0.0;
        const double a = sound_speed(P, c);
        for (int d = 0; d < L.dim; ++d) {
            const double v = L.dx[d] / (a + fabs(st[(L.A_VEL + d) * L.N + g]));
            if (v < mn) mn = v;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_down_sync(0xffffffffu, mn, o);
        if (w < mn) mn = w;
    }
    __shared__ double red[kNaThreads / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mn;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = red[0];
        for (int w = 1; w < kNaThreads / 32; ++w)
            if (red[w] < b) b = red[w];
        scratch[blockIdx.x] = b;
    }
}

__global__ void k_na_cfl_final(int nblocks, double cfl, double* scratch)
{
    double mn = 1.79769313486231570815e+308;
    for (int b = threadIdx.x; b < nblocks; b += kNaThreads)
        if (scratch[b] < mn) mn = scratch[b];
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_down_sync(0xffffffffu, mn, o);
        if (w < mn) mn = w;
    }
    __shared__ double red[kNaThreads / 32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mn;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = red[0];
        for (int w = 1; w < kNaThreads / 32; ++w)
            if (red[w] < b) b = red[w];
        scratch[kNaMaxBlocks] = cfl * b;
    }
}

// Device address of the scratch array, per device, looked up once.
constexpr int kNaMaxDevices = 64;
std::mutex g_na_mutex;
double* g_na_addr[kNaMaxDevices] = {nullptr};

double* scratch_for_current_device()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, tj_noalloc_scratch);
        if (e != cudaSuccess) {
            std::fprintf(stderr, "tj_compute_dt_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return nullptr;
        }
        g_na_addr[dev] = (double*)p;
    }
    return g_na_addr[dev];
}

}  // namespace
}  // namespace tj

using namespace tj;

extern "C" int tj_compute_dt_noalloc(const tj_params* p, const int* n_cells, const double* dim_l, const double* state,
                                     double* dt, void* stream)
{
    if (!p || !n_cells || !dim_l || !state || !dt) return TJ_ERR_ARG;
    if (p->dim < 1 || p->dim > 3 || p->n_materials < 1 || p->n_materials > TJ_MAX_MATERIALS || p->n_mixtures != 0) {
        std::fprintf(stderr, "tj_compute_dt_noalloc: unsupported parameters\n");
        return TJ_ERR_ARG;
    }
    // The same component offsets as the context's (AccessPattern order).
    DevParams P;
    make_layouts(*p, P);
    NaLayout L;
    L.M = P.M;
    L.dim = P.dim;
    L.solid = P.solid;
    L.cfl = P.cfl;
    L.N = 1;
    for (int d = 0; d < 3; ++d) {
        L.n[d] = d < p->dim ? n_cells[d] : 1;
        // each extent and the running product stay within the maximum, so the
        // product never overflows
        if (L.n[d] < 1 || L.n[d] > TJ_NOALLOC_MAX_CELLS || L.N * L.n[d] > TJ_NOALLOC_MAX_CELLS) {
            std::fprintf(stderr,
                         "tj_compute_dt_noalloc: domain extent %d along axis %d is not positive or exceeds the maximum "
                         "of %d cells (TJ_NOALLOC_MAX_CELLS)\n",
                         L.n[d], d, TJ_NOALLOC_MAX_CELLS);
            return TJ_ERR_ARG;
        }
        L.dx[d] = (d < p->dim ? dim_l[d] : 1.0) / (double)L.n[d];
        L.N *= L.n[d];
    }
    L.A_ALPHA = P.A_ALPHA;
    L.A_ARHO = P.A_ARHO;
    L.A_RHOK = P.A_RHOK;
    L.A_RHO = P.A_RHO;
    L.A_VEL = P.A_VEL;
    L.A_P = P.A_P;
    L.A_HJ2 = P.A_HJ2;
    double* scratch = scratch_for_current_device();
    if (!scratch) return TJ_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    int nb = (int)((L.N + kNaCellsPerBlock - 1) / kNaCellsPerBlock);
    double cfl = L.cfl;
    // cudaLaunchKernel reports this launch's own failure, and leaves any error
    // that earlier, unrelated work left pending to its owner
    void* a1[] = {&P, &L, &state, &scratch};
    if (cudaLaunchKernel((const void*)k_na_cfl_partial, dim3(nb), dim3(kNaThreads), a1, 0, st) != cudaSuccess)
        return TJ_ERR_CUDA;
    void* a2[] = {&nb, &cfl, &scratch};
    if (cudaLaunchKernel((const void*)k_na_cfl_final, dim3(1), dim3(kNaThreads), a2, 0, st) != cudaSuccess)
        return TJ_ERR_CUDA;
    if (cudaMemcpyAsync(dt, scratch + kNaMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return TJ_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return TJ_ERR_CUDA;
    return TJ_OK;
}
