// Binary32 instance of the per-direction kernels (tj_path.cuh) behind the
// fused-state interface: the mixed precision of every configuration the fused
// kernels do not cover (1-D; solids with the 5-wave solver, plasticity and
// cleanUpV; several 2-D domains). The state is binary32 with the total energy
// as a compensated pair; the pressure closure is evaluated in binary64 (the
// radial-return yield projection in binary64 gave the same accuracy, at 41 %
// more time per copper step); the CFL minimum is a pass over the state at the
// start of each step, as in the binary64 path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "tj_mixed.cuh"
#include "tj_path.cuh"
#include "tj_path_launch.cuh"

namespace tj {

namespace {

constexpr int kT32 = 256;

inline int nb32(long long n, int cap = 152 * 16)
{
    long long b = (n + kT32 - 1) / kT32;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

// binary64 carried state (+ THINC scratch) -> binary32, the energy split into (hi, lo)
__global__ void k_to32(DevParams32 P, PathBufs<float> b, const double* A, const double* uls, const double* urs,
                       const double* gs0, const double* gs1, const double* gs2)
{
    const long long nt = b.ntot;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        for (int w = 0; w < P.d.NS; ++w) b.A[w * nt + g] = (float)A[w * nt + g];
        const double E = A[P.S_E * nt + g];
        const float eh = (float)E;
        b.A[P.S_E * nt + g] = eh;
        b.A[P.S_ELO * nt + g] = (float)(E - (double)eh);
        if (uls)
            for (int m = 0; m < P.M; ++m) {
                b.ulstar[(long long)m * nt + g] = (float)uls[(long long)m * nt + g];
                b.urstar[(long long)m * nt + g] = (float)urs[(long long)m * nt + g];
            }
    }
    const double* gsrc[3] = {gs0, gs1, gs2};
    for (int d = 0; d < P.dim; ++d) {
        if (!gsrc[d]) continue;
        const long long nf = (long long)P.M * b.nftot[d];
        for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x)
            b.gstar[d][f] = (float)gsrc[d][f];
    }
}

__global__ void k_to64(DevParams32 P, PathBufs<float> b, double* A)
{
    const long long nt = b.ntot;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        for (int w = 0; w < P.d.NS; ++w) A[w * nt + g] = b.A[w * nt + g];
        A[P.S_E * nt + g] = (double)b.A[P.S_E * nt + g] + (double)b.A[P.S_ELO * nt + g];
    }
}

__global__ void k_reset_dtmin32(DevScalars* s)
{
    if (threadIdx.x == 0) s->dtmin_bits = 0x7FEFFFFFFFFFFFFFull;
}

struct General32 : MixedBase {
    DevParams32 P;
    PathBufs<float> b;
    float *A = nullptr, *B = nullptr, *C = nullptr, *UL = nullptr, *UR = nullptr, *FX = nullptr;
    float *uls = nullptr, *urs = nullptr, *gs[3] = {nullptr, nullptr, nullptr};
    int ns32 = 0;

    ~General32() override
    {
        float* ps[] = {A, B, C, UL, UR, FX, uls, urs, gs[0], gs[1], gs[2]};
        for (float* p : ps)
            if (p) cudaFree(p);
    }

    int alloc(const DevParams& DP, long long ntot, const long long* nftot, cudaStream_t st)
    {
        P = make_params32(DP);
        ns32 = DP.NS + 1;
        const size_t nt = (size_t)ntot;
        size_t fmax = (size_t)std::max(nftot[0], std::max(nftot[1], nftot[2]));
        auto al = [&](float** p, size_t n) {
            if (cudaMalloc(p, sizeof(float) * std::max<size_t>(n, 1)) != cudaSuccess) return false;
            cudaMemsetAsync(*p, 0, sizeof(float) * std::max<size_t>(n, 1), st);
            return true;
        };
        bool ok = al(&A, ns32 * nt) && al(&B, ns32 * nt) && al(&C, ns32 * nt) && al(&UL, DP.NF * nt) &&
                  al(&UR, DP.NF * nt) && al(&FX, DP.NX * fmax);
        if (ok && DP.thinc) {
            ok = al(&uls, DP.M * nt) && al(&urs, DP.M * nt);
            for (int d = 0; ok && d < DP.dim; ++d) ok = al(&gs[d], DP.M * (size_t)nftot[d]);
        }
        if (!ok) return TJ_ERR_CUDA;
        b.A = A;
        b.B = B;
        b.C = C;
        b.UL = UL;
        b.UR = UR;
        b.FX = FX;
        b.ulstar = uls;
        b.urstar = urs;
        for (int d = 0; d < 3; ++d) {
            b.gstar[d] = gs[d];
            b.nftot[d] = nftot[d];
        }
        b.ntot = ntot;
        return TJ_OK;
    }

    // geometry pointers are the binary64 context's
    void sync_geometry(const Fp64Bufs& fb)
    {
        b.cell_box = fb.cell_box;
        b.boxes = fb.boxes;
        b.doms = fb.doms;
        b.scal = fb.scal;
        b.ndom = fb.ndom;
    }

    int set_boxes(const std::vector<DevDomain>&, const std::vector<std::vector<int>>&, cudaStream_t) override
    {
        return TJ_OK;
    }

    int from_fp64(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st) override
    {
        (void)DP;
        sync_geometry(fb);
        k_to32<<<nb32(b.ntot), kT32, 0, st>>>(P, b, fb.A, fb.ulstar, fb.urstar, fb.gstar[0], fb.gstar[1], fb.gstar[2]);
        return 1;
    }

    int to_fp64(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st) override
    {
        (void)DP;
        sync_geometry(fb);
        k_to64<<<nb32(b.ntot), kT32, 0, st>>>(P, b, fb.A);
        return 1;
    }

    int cfl(const Fp64Bufs& fb, cudaStream_t st) override
    {
        sync_geometry(fb);
        k_reset_dtmin32<<<1, 32, 0, st>>>(fb.scal);
        return 1 + path_cfl_any(P, b, (const float*)A, st, nullptr);
    }

    int stage(const float* X, float* Y, int finish, cudaStream_t st, Prof* pr)
    {
        int n = 0;
        for (int d = 0; d < P.dim; ++d) n += path_dir_any(P, b, X, Y, d, d == 0, d == P.dim - 1, finish, st, pr);
        return n;
    }

    int step(const DevParams& DP, const Fp64Bufs& fb, cudaStream_t st, Prof* pr) override
    {
        sync_geometry(fb);
        int n = 0;
        n += path_cfl_any(P, b, (const float*)A, st, pr);
        n += fp64_dt_finalize(DP, fb, 1, st);
        n += stage(A, B, 0, st, pr);
        n += stage(B, C, 1, st, pr);
        n += fp64_step_end(fb, st);
        return n;
    }

    void describe(char* buf, size_t len) const override
    {
        std::snprintf(buf, len, "binary32 per-direction kernels (%d-D), binary64 pressure closure and plastic return map", P.dim);
    }
};

}  // namespace

DevParams32 make_params32(const DevParams& DP)
{
    DevParams32 P;
    std::memset(&P, 0, sizeof P);
    P.d = DP;
    for (int m = 0; m < TJ_MAX_MAT; ++m) {
        P.rG[m] = (m < DP.M && DP.prm[m][0] != 1.0) ? 1.0 / (DP.prm[m][0] - 1.0) : 0.0;
        P.rR0h[m] = (m < DP.M && DP.prm[m][4] != 0.0) ? 0.5 / DP.prm[m][4] : 0.0;
    }
    P.dim = DP.dim;
    P.M = DP.M;
    P.solid = DP.solid;
    P.thinc = DP.thinc;
    P.plastic = DP.plastic;
    P.muscl = DP.muscl;
    P.any_solid = DP.any_solid;
    P.radial = DP.radial;
    P.nmix = DP.nmix;
    P.reactive = DP.reactive;
    for (int d = 0; d < 3; ++d) {
        P.lo_bc[d] = DP.lo_bc[d];
        P.hi_bc[d] = DP.hi_bc[d];
    }
    P.cfl = (float)DP.cfl;
    P.beta = (float)DP.beta;
    for (int m = 0; m < TJ_MAX_MAT; ++m) {
        P.phase[m] = DP.phase[m];
        P.eos[m] = DP.eos[m];
        P.yield[m] = (float)DP.yield[m];
        for (int k = 0; k < TJ_MAX_EOS_PARAMS; ++k) P.prm[m][k] = (float)DP.prm[m][k];
    }
#define CP(f) P.f = DP.f
    CP(S_ALPHA); CP(S_ARHO); CP(S_RHOK); CP(S_RHO); CP(S_RHOU); CP(S_VEL); CP(S_E); CP(S_P); CP(S_V); CP(S_HJ2);
    CP(S_EPS); CP(S_ARE); CP(S_RMIX); CP(S_LAM); CP(S_ARL); CP(F_ARL); CP(X_ARL);
    CP(F_ALPHA); CP(F_ARHO); CP(F_RHO); CP(F_RHOU); CP(F_VEL); CP(F_E); CP(F_P); CP(F_A); CP(F_SIGMA); CP(F_V);
    CP(F_ARE); CP(NF);
    CP(X_ALPHA); CP(X_ARHO); CP(X_RHOU); CP(X_E); CP(X_SSTAR); CP(X_V); CP(X_VSTAR); CP(X_ARE); CP(NX);
#undef CP
    P.S_ELO = DP.NS;  // the low word of the energy after the binary64 layout
    P.NS = DP.NS + 1;
    return P;
}

MixedBase* general32_create(const DevParams& DP, long long ntot, const long long* nftot, cudaStream_t st, int* err)
{
    auto* m = new General32();
    *err = m->alloc(DP, ntot, nftot, st);
    return m;
}

}  // namespace tj
