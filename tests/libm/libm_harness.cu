// Test harness (not part of the library): evaluates the project-written
// binary64 transcendentals of tenjin_gb300/csrc/tj_math.cuh and CUDA's own
// functions on the same arguments on the GPU, so that the tests can compare
// them with each other, with the oracle's host build of the same algorithms
// and with the host libm.
#include <cuda_runtime.h>

#include "tj_math.cuh"

using namespace tj;

// fn: 0 exp, 1 log, 2 pow, 3 cosh, 4 tanh, 5 expm1
__global__ void k_eval(int fn, const double* x, const double* y, int n, double* ours, double* cuda)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double a = x[i], b = y[i];
        double o = 0.0, c = 0.0;
        switch (fn) {
            case 0: o = tjm_exp(a); c = exp(a); break;
            case 1: o = tjm_log(a); c = log(a); break;
            case 2: o = tjm_pow(a, b); c = pow(a, b); break;
            case 3: o = tjm_cosh(a); c = cosh(a); break;
            case 4: o = tjm_tanh(a); c = tanh(a); break;
            case 5: o = tjm_expm1(a); c = expm1(a); break;
            default: break;
        }
        ours[i] = o;
        cuda[i] = c;
    }
}

extern "C" int tjm_eval_gpu(int fn, const double* x, const double* y, int n, double* ours, double* cuda)
{
    double* d = nullptr;
    const size_t bytes = sizeof(double) * (size_t)n;
    if (cudaMalloc(&d, 4 * bytes) != cudaSuccess) return -1;
    cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(d + n, y, bytes, cudaMemcpyHostToDevice);
    k_eval<<<(n + 255) / 256, 256>>>(fn, d, d + n, n, d + 2 * (size_t)n, d + 3 * (size_t)n);
    cudaError_t e = cudaGetLastError();
    cudaMemcpy(ours, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
    cudaMemcpy(cuda, d + 3 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(d);
    return e == cudaSuccess ? 0 : -2;
}
