// Tangent-linear (forward-mode) run of the FP64 update: the per-direction
// kernels instantiated with Dual values (tj_dual.cuh) carry one directional
// derivative of every word through the same steps as the FP64 path, from the
// initial primitives (primitiveToConservative, initialise.cpp:111-123) over
// nsteps steps of advance with the post-advance operators (main.cpp:145-187),
// dt frozen. The values are the FP64 path's own, bit for bit; the directions
// are exact derivatives of the branch the FP64 run takes, for every
// configuration that path covers except mixtures (the mixture EOS's root
// find): 1-, 2- and 3-D, fluids and solids, the 5-wave solver, the plastic
// radial return, cleanUpV, the radial source, BVD-THINC with its scratch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "tj_dual.cuh"
#include "tj_dual_path.cuh"
#include "tj_path.cuh"
#include "tj_path_launch.cuh"
#include "tj_tangent.cuh"

namespace tj {

namespace {

constexpr int kT = 256;

inline int nbt(long long n)
{
    long long b = (n + kT - 1) / kT;
    return (int)std::max(1LL, std::min(b, 152LL * 16));
}

// The initial state of one domain from its primitives and their directions
// (the tj_set_primitive layout, k_prim_to_state's closure).
__global__ void k_t_prim_to_state(DevParamsT P, PathBufs<Dual> b, int dom, const double* prim, const double* dprim,
                                  Dual* X)
{
    const long long nt = b.ntot;
    const DevDomain D = b.doms[dom];
    const long long nd = (long long)D.n[0] * D.n[1] * D.n[2];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nd; t += (long long)gridDim.x * blockDim.x) {
        CellT<Dual> c;
        int w = 0;
        auto in = [&]() {
            const Dual x(prim[w * nd + t], dprim ? dprim[w * nd + t] : 0.0);
            ++w;
            return x;
        };
        for (int m = 0; m < P.M; ++m) c.alpha[m] = in();
        for (int m = 0; m < P.M; ++m) c.rhok[m] = in();
        for (int r = 0; r < 3; ++r) c.vel[r] = in();
        c.p = in();
        c.hj2 = Dual(0.0);
        if (P.solid)
            for (int qq = 0; qq < 9; ++qq) c.V[qq] = in();
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) c.eps[m] = in();
        p2c(P, c);
        store_state(P, X, nt, D.off + t, c);
    }
}

// Values and directions of the carried words of one domain into the
// AccessPattern layout of tj_download_domain (ap: values, dap: directions);
// components derived from the carried words (sound speed, USTAR, sigma,
// VSTAR, devH) are left zero.
__global__ void k_t_state_to_ap(DevParamsT P, PathBufs<Dual> b, int dom, const Dual* X, const int* a_to_s, int ncomp,
                                double* ap, double* dap)
{
    const long long nt = b.ntot;
    const DevDomain D = b.doms[dom];
    const long long nd = (long long)D.n[0] * D.n[1] * D.n[2];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nd; t += (long long)gridDim.x * blockDim.x)
        for (int a = 0; a < ncomp; ++a) {
            const int s = a_to_s[a];
            const Dual x = s >= 0 ? X[(long long)s * nt + D.off + t] : Dual(0.0);
            if (ap) ap[a * nd + t] = x.v;
            dap[a * nd + t] = x.d;
        }
}

__global__ void k_t_set_dt(DevScalars* s, double dt)
{
    if (threadIdx.x == 0) {
        s->dt = dt;
        s->done = 0;
    }
}

// One direction of one stage: the instances with two materials along x and
// y, the generic instance otherwise.
int tdir(const DevParamsT& P, const PathBufs<Dual>& b, const Dual* X, Dual* Y, int d, int first, int last, int finish,
         cudaStream_t st)
{
    if (P.M == 2 && d == 0)
        return path_dir<WithM<DevParamsT, 2>, 0>(WithM<DevParamsT, 2>(P), b, X, Y, d, first, last, finish, st, nullptr);
    if (P.M == 2 && d == 1)
        return path_dir<WithM<DevParamsT, 2>, 1>(WithM<DevParamsT, 2>(P), b, X, Y, d, first, last, finish, st, nullptr);
    return path_dir<DevParamsT, -1>(P, b, X, Y, d, first, last, finish, st, nullptr);
}

int tstage(const DevParamsT& P, const PathBufs<Dual>& b, const Dual* X, Dual* Y, int finish, cudaStream_t st)
{
    int n = 0;
    for (int d = 0; d < P.dim; ++d) n += tdir(P, b, X, Y, d, d == 0, d == P.dim - 1, finish, st);
    return n;
}

}  // namespace

struct TanState {
    Dual *A = nullptr, *B = nullptr, *C = nullptr, *UL = nullptr, *UR = nullptr, *FX = nullptr;
    Dual *uls = nullptr, *urs = nullptr, *gs[3] = {nullptr, nullptr, nullptr};
    size_t cap[11] = {};  // words held by A, B, C, UL, UR, FX, uls, urs, gs[0..2]
    DevScalars* scal = nullptr;
    int* a_to_s = nullptr;
};

TanState* tan_create() { return new TanState(); }

void tan_destroy(TanState* t)
{
    if (!t) return;
    void* ps[] = {t->A, t->B, t->C, t->UL, t->UR, t->FX, t->uls, t->urs, t->gs[0], t->gs[1], t->gs[2], t->scal, t->a_to_s};
    for (void* p : ps)
        if (p) cudaFree(p);
    delete t;
}

namespace {

bool grow(Dual** p, size_t& cap, size_t n)
{
    n = std::max<size_t>(n, 1);
    if (*p && cap >= n) return true;
    if (*p) cudaFree(*p);
    *p = nullptr;
    cap = 0;
    if (cudaMalloc(p, sizeof(Dual) * n) != cudaSuccess) return false;
    cap = n;
    return true;
}

DevParamsT make_params_t(const DevParams& D, const double* deos)
{
    DevParamsT P;
    std::memset(&P, 0, sizeof P);
    P.dim = D.dim; P.M = D.M; P.solid = D.solid; P.thinc = D.thinc; P.plastic = D.plastic; P.muscl = D.muscl;
    P.any_solid = D.any_solid; P.fused64 = 0; P.radial = D.radial; P.nmix = D.nmix; P.reactive = D.reactive;
    for (int d = 0; d < 3; ++d) {
        P.lo_bc[d] = D.lo_bc[d];
        P.hi_bc[d] = D.hi_bc[d];
    }
    P.cfl = Dual(D.cfl);
    P.beta = Dual(D.beta);
    for (int m = 0; m < TJ_MAX_MAT; ++m) {
        P.phase[m] = D.phase[m];
        P.eos[m] = D.eos[m];
        P.yield[m] = Dual(D.yield[m]);
        for (int k = 0; k < TJ_MAX_EOS_PARAMS; ++k)
            P.prm[m][k] = Dual(D.prm[m][k], (deos && m < D.M) ? deos[m * TJ_MAX_EOS_PARAMS + k] : 0.0);
    }
#define CP(f) P.f = D.f
    CP(S_ALPHA); CP(S_ARHO); CP(S_RHOK); CP(S_RHO); CP(S_RHOU); CP(S_VEL); CP(S_E); CP(S_P); CP(S_V); CP(S_HJ2);
    CP(S_EPS); CP(S_ARE); CP(NS); CP(S_RMIX); CP(S_LAM); CP(S_ARL);
    CP(F_ALPHA); CP(F_ARHO); CP(F_RHO); CP(F_RHOU); CP(F_VEL); CP(F_E); CP(F_P); CP(F_A); CP(F_SIGMA); CP(F_V);
    CP(F_ARE); CP(NF); CP(F_ARL);
    CP(X_ALPHA); CP(X_ARHO); CP(X_RHOU); CP(X_E); CP(X_SSTAR); CP(X_V); CP(X_VSTAR); CP(X_ARE); CP(NX); CP(X_ARL);
#undef CP
    P.S_ELO = -1;
    return P;
}

}  // namespace

long long tan_run(TanState* t, const DevParams& DP, const Fp64Bufs& fb, int dom, const double* prim,
                  const double* dprim, const double* deos, int nsteps, const double* dt, double* ap, double* dap,
                  cudaStream_t st)
{
    if (!t || nsteps < 1) return TJ_ERR_ARG;
    const DevParamsT P = make_params_t(DP, deos);
    const size_t nt = (size_t)fb.ntot;
    size_t fmax = (size_t)std::max(fb.nftot[0], std::max(fb.nftot[1], fb.nftot[2]));
    bool ok = grow(&t->A, t->cap[0], DP.NS * nt) && grow(&t->B, t->cap[1], DP.NS * nt) &&
              grow(&t->C, t->cap[2], DP.NS * nt) && grow(&t->UL, t->cap[3], DP.NF * nt) &&
              grow(&t->UR, t->cap[4], DP.NF * nt) && grow(&t->FX, t->cap[5], DP.NX * fmax);
    if (ok && DP.thinc) {
        ok = grow(&t->uls, t->cap[6], DP.M * nt) && grow(&t->urs, t->cap[7], DP.M * nt);
        for (int d = 0; ok && d < DP.dim; ++d) ok = grow(&t->gs[d], t->cap[8 + d], DP.M * (size_t)fb.nftot[d]);
    }
    if (ok && !t->scal) ok = cudaMalloc(&t->scal, sizeof(DevScalars)) == cudaSuccess;
    if (ok && !t->a_to_s) ok = cudaMalloc(&t->a_to_s, sizeof(int) * 64) == cudaSuccess;
    if (!ok) return TJ_ERR_CUDA;
    // AccessPattern component -> carried word (-1: derived)
    int a2s[64];
    for (int a = 0; a < 64; ++a) a2s[a] = -1;
    auto map = [&](int a0, int s0, int n) {
        if (a0 >= 0 && s0 >= 0)
            for (int k = 0; k < n; ++k) a2s[a0 + k] = s0 + k;
    };
    map(DP.A_ALPHA, DP.S_ALPHA, DP.M);
    map(DP.A_ARHO, DP.S_ARHO, DP.M);
    map(DP.A_RHOK, DP.S_RHOK, DP.M);
    map(DP.A_RHO, DP.S_RHO, 1);
    map(DP.A_RHOU, DP.S_RHOU, 3);
    map(DP.A_VEL, DP.S_VEL, 3);
    map(DP.A_E, DP.S_E, 1);
    map(DP.A_P, DP.S_P, 1);
    if (DP.solid) {
        map(DP.A_V, DP.S_V, 9);
        map(DP.A_HJ2, DP.S_HJ2, 1);
    }
    if (DP.plastic) {
        map(DP.A_EPS, DP.S_EPS, DP.M);
        map(DP.A_ARE, DP.S_ARE, DP.M);
    }
    if (DP.NCOMP > 64) return TJ_ERR_ARG;
    cudaMemcpyAsync(t->a_to_s, a2s, sizeof(int) * DP.NCOMP, cudaMemcpyHostToDevice, st);

    PathBufs<Dual> b;
    b.A = t->A;
    b.B = t->B;
    b.C = t->C;
    b.UL = t->UL;
    b.UR = t->UR;
    b.FX = t->FX;
    b.ulstar = t->uls;
    b.urstar = t->urs;
    for (int d = 0; d < 3; ++d) {
        b.gstar[d] = t->gs[d];
        b.nftot[d] = fb.nftot[d];
    }
    b.cell_box = fb.cell_box;
    b.boxes = fb.boxes;
    b.doms = fb.doms;
    b.scal = t->scal;
    b.ntot = fb.ntot;
    b.ndom = fb.ndom;
    long long n = 0;
    cudaMemsetAsync(t->scal, 0, sizeof(DevScalars), st);
    // a fresh start: the whole state zero (other domains), THINC scratch zero
    cudaMemsetAsync(t->A, 0, sizeof(Dual) * DP.NS * nt, st);
    if (DP.thinc) {
        cudaMemsetAsync(t->uls, 0, sizeof(Dual) * DP.M * nt, st);
        cudaMemsetAsync(t->urs, 0, sizeof(Dual) * DP.M * nt, st);
        for (int d = 0; d < DP.dim; ++d) cudaMemsetAsync(t->gs[d], 0, sizeof(Dual) * DP.M * fb.nftot[d], st);
    }
    k_t_prim_to_state<<<nbt(fb.ntot), kT, 0, st>>>(P, b, dom, prim, dprim, t->A);
    ++n;
    for (int s = 0; s < nsteps; ++s) {
        k_t_set_dt<<<1, 32, 0, st>>>(t->scal, dt[s]);
        n += 1 + tstage(P, b, t->A, t->B, 0, st);
        n += tstage(P, b, t->B, t->C, 1, st);
    }
    k_t_state_to_ap<<<nbt(fb.ntot), kT, 0, st>>>(P, b, dom, t->A, t->a_to_s, DP.NCOMP, ap, dap);
    return n + 1;
}

// The status word of the last tangent run (TJ_OK or the first error a kernel
// raised).
int tan_status(TanState* t, int* status, cudaStream_t st)
{
    DevScalars s;
    if (cudaMemcpyAsync(&s, t->scal, sizeof s, cudaMemcpyDeviceToHost, st) != cudaSuccess) return TJ_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return TJ_ERR_CUDA;
    *status = s.status;
    return TJ_OK;
}

}  // namespace tj
