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
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "tj_device.cuh"
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
    NaLayout L;
    L.M = p->n_materials;
    L.dim = p->dim;
    L.solid = p->SOLID;
    L.cfl = p->CFL;
    L.N = 1;
    for (int d = 0; d < 3; ++d) {
        L.n[d] = d < p->dim ? n_cells[d] : 1;
        if (L.n[d] < 1) return TJ_ERR_ARG;
        L.dx[d] = (d < p->dim ? dim_l[d] : 1.0) / (double)L.n[d];
        L.N *= L.n[d];
    }
    if (L.N > TJ_NOALLOC_MAX_CELLS) {
        std::fprintf(stderr, "tj_compute_dt_noalloc: %lld cells exceed the maximum of %d (TJ_NOALLOC_MAX_CELLS)\n", L.N,
                     TJ_NOALLOC_MAX_CELLS);
        return TJ_ERR_ARG;
    }
    // AccessPattern offsets (accesspattern.cpp:44-79)
    const int M = L.M;
    L.A_ALPHA = 0;
    L.A_ARHO = M;
    L.A_RHOK = 2 * M;
    L.A_RHO = 3 * M;
    L.A_VEL = 3 * M + 4;
    L.A_P = 3 * M + 8;
    L.A_HJ2 = 3 * M + 11 + 9 + 27;
    DevParams P;
    std::memset(&P, 0, sizeof P);
    P.dim = p->dim;
    P.M = M;
    P.solid = p->SOLID;
    for (int m = 0; m < M; ++m) {
        P.phase[m] = p->materials[m].phase;
        P.eos[m] = p->materials[m].eos;
        for (int q = 0; q < TJ_MAX_EOS_PARAMS; ++q)
            P.prm[m][q] = q < p->materials[m].nparams ? p->materials[m].params[q] : 0.0;
        if (P.phase[m] == TJ_PHASE_SOLID) P.any_solid = 1;
    }
    double* scratch = scratch_for_current_device();
    if (!scratch) return TJ_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    const int nb = (int)((L.N + kNaCellsPerBlock - 1) / kNaCellsPerBlock);
    k_na_cfl_partial<<<nb, kNaThreads, 0, st>>>(P, L, state, scratch);
    k_na_cfl_final<<<1, kNaThreads, 0, st>>>(nb, L.cfl, scratch);
    if (cudaGetLastError() != cudaSuccess) return TJ_ERR_CUDA;
    if (cudaMemcpyAsync(dt, scratch + kNaMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return TJ_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return TJ_ERR_CUDA;
    return TJ_OK;
}
