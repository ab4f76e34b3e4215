// FP64 reference-faithful kernels of Tenjin's per-timestep update.
//
// One RK stage (HLLCadvance, hllc.cpp:579-695) is, per direction d:
//   k_recon   per cell : MUSCL (hllc.cpp:541-575), BVD-THINC (thinc.cpp:67-208),
//                        cleanUpAlpha of the reconstructed states (hllc.cpp:628-629),
//                        primitiveToConservative + getSoundSpeed (634-638)
//   k_flux    per face : HLLC (hllc.cpp:384-487) or 5-wave (133-380)
//   k_update  per cell : update (hllc.cpp:493-523); after the last direction
//                        conservativeToPrimitive (689), and at the end of the
//                        second stage the RK2 average (705), plasticUpdate,
//                        cleanUpV, cleanUpAlpha and the NaN check
//                        (main.cpp:145-187).
// Ghost cells are never stored: a read outside a domain maps the index back
// (foextrap: nearest cell; reflect: mirror, negating the normal velocity and
// momentum), which is what the reference's FillDomainBoundary and
// FillBoundary calls leave in the ghost cells (main.cpp:124-126,
// hllc.cpp:642-646,690-691).
#include <cuda_runtime.h>

#include "tj_path.cuh"
#include "tj_path_launch.cuh"

namespace tj {

static constexpr int kThreads = 256;

static inline int nblocks(long long n, int cap = 152 * 16)
{
    long long b = (n + kThreads - 1) / kThreads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}


__global__ void k_dt_finalize(DevParams P, DevScalars* s, int clamp)
{
    if (threadIdx.x != 0) return;
    double raw = __longlong_as_double((long long)s->dtmin_bits);
    s->dtmin_raw = raw;
    s->dtmin_bits = 0x7FEFFFFFFFFFFFFFull;
    if (!clamp) return;
    if (s->done) return;
    if (!(s->t < s->t_end)) { s->done = 1; return; }
    double dt = P.cfl * raw;
    if (s->t + dt > s->t_end) dt = s->t_end - s->t;
    if (s->n < 5) dt *= 0.2;
    s->dt = dt;
}

__global__ void k_step_end(DevScalars* s)
{
    if (threadIdx.x != 0 || s->done) return;
    if (s->nan_flag) {
        s->done = 1;
        atomicCAS(&s->status, 0, TJ_ERR_NAN);
        return;
    }
    s->t += s->dt;
    s->n += 1;
}

__global__ void k_set_dt(DevScalars* s, double dt)
{
    if (threadIdx.x != 0) return;
    s->dt = dt;
    s->done = 0;
}

// ---------------------------------------------------------------------------
// Whole-array cell operators of the C ABI.
// ---------------------------------------------------------------------------
__global__ void k_cell_op(DevParams P, Fp64Bufs b, double* X, const double* X2, int op, double dt)
{
    const long long nt = b.ntot;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nt; g += (long long)gridDim.x * blockDim.x) {
        CellS c;
        load_state(P, X, nt, g, nullptr, c);
        if (P.solid && (op == OP_P2C)) {
            // the primitive list carries V; HJ2 recomputed by p2c
        }
        switch (op) {
            case OP_C2P: {
                int e = c2p(P, c);
                if (e) set_status(b.scal, e);
                break;
            }
            case OP_REACTIVE: {
                int e = reactive_cell(P, c, dt);
                if (e) set_status(b.scal, e);
                break;
            }
            case OP_P2C: p2c(P, c); break;
            case OP_CLEAN_ALPHA: {
                int e = cleanup_alpha(P, c.alpha);
                if (e) set_status(b.scal, e);
                break;
            }
            case OP_CLEAN_V: cleanup_v_cell(P, c); break;
            case OP_PLASTIC: {
                int e = plastic_cell(P, c);
                if (e) set_status(b.scal, e);
                c2p(P, c);
                break;
            }
            case OP_RADIAL: {
                // geometricSourceTerm (radial.cpp:37-54) with the stress of
                // the state as its last conservativeToPrimitive left it
                const DevDomain D = b.doms[find_dom(b.doms, b.ndom, g)];
                hencky(P, c);
                stress(P, c);
                double sg[9];
                for (int q = 0; q < 9; ++q) sg[q] = c.sigma[q];
                radial_source(P, c, sg, (int)((g - D.off) % D.n[0]), D.dx[0], dt);
                int e = c2p(P, c);
                if (e) set_status(b.scal, e);
                break;
            }
            case OP_NAN: {
                const int q = find_dom(b.doms, b.ndom, g);
                if (b.cell_box[g] == b.doms[q].nbox - 1 && cell_has_nan(P, c)) atomicOr(&b.scal->nan_flag, 1);
                continue;
            }
            default: break;
        }
        store_state(P, X, nt, g, c);
    }
}

// AccessPattern blocks <-> carried state, for one box of one domain. The AP
// array is indexed ap[n*cstride + (i+go) + ld_i*((j+go) + ld_j*(k+go))] for box
// cell (i,j,k) relative to the box lo, where go is the ghost offset.
__global__ void k_ap_to_state(DevParams P, Fp64Bufs b, int dom, int lx, int ly, int lz, int nx, int ny, int nz,
                              const double* ap, int ld_i, int ld_j, long long cs, int go, double* X)
{
    const long long nt = b.ntot, nb = (long long)nx * ny * nz;
    const DevDomain D = b.doms[dom];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nb; t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / ((long long)nx * ny));
        long long src = (i + go) + (long long)ld_i * ((j + (P.dim > 1 ? go : 0)) + (long long)ld_j * (k + (P.dim > 2 ? go : 0)));
        long long g = D.off + (lx + i) + (long long)D.n[0] * ((ly + j) + (long long)D.n[1] * (lz + k));
#define APV(comp) ap[(long long)(comp)*cs + src]
        for (int m = 0; m < P.M; ++m) {
            X[(P.S_ALPHA + m) * nt + g] = APV(P.A_ALPHA + m);
            X[(P.S_ARHO + m) * nt + g] = APV(P.A_ARHO + m);
            X[(P.S_RHOK + m) * nt + g] = APV(P.A_RHOK + m);
        }
        X[P.S_RHO * nt + g] = APV(P.A_RHO);
        for (int r = 0; r < 3; ++r) {
            X[(P.S_RHOU + r) * nt + g] = APV(P.A_RHOU + r);
            X[(P.S_VEL + r) * nt + g] = APV(P.A_VEL + r);
        }
        X[P.S_E * nt + g] = APV(P.A_E);
        X[P.S_P * nt + g] = APV(P.A_P);
        if (P.solid) {
            for (int qq = 0; qq < 9; ++qq) X[(P.S_V + qq) * nt + g] = APV(P.A_V + qq);
            X[P.S_HJ2 * nt + g] = APV(P.A_HJ2);
        }
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) {
                X[(P.S_EPS + m) * nt + g] = APV(P.A_EPS + m);
                X[(P.S_ARE + m) * nt + g] = APV(P.A_ARE + m);
            }
        if (P.nmix) {
            X[P.S_RMIX * nt + g] = APV(P.A_RMIX);
            X[(P.S_RMIX + 1) * nt + g] = APV(P.A_RMIX + 1);
            X[P.S_LAM * nt + g] = APV(P.A_LAM);
            X[P.S_ARL * nt + g] = APV(P.A_ARL);
        }
#undef APV
    }
}

__global__ void k_state_to_ap(DevParams P, Fp64Bufs b, int dom, int lx, int ly, int lz, int nx, int ny, int nz,
                              const double* X, double* ap, int ld_i, int ld_j, long long cs, int go, long long t0,
                              long long t1)
{
    const long long nt = b.ntot;
    const DevDomain D = b.doms[dom];
    for (long long t = t0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; t < t1; t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % nx), j = (int)((t / nx) % ny), k = (int)(t / ((long long)nx * ny));
        long long dst = (i + go) + (long long)ld_i * ((j + (P.dim > 1 ? go : 0)) + (long long)ld_j * (k + (P.dim > 2 ? go : 0)));
        long long g = D.off + (lx + i) + (long long)D.n[0] * ((ly + j) + (long long)D.n[1] * (lz + k));
        CellS c;
        load_state(P, X, nt, g, nullptr, c);
        // Derived components: Hencky strain and stress of the carried state,
        // sound speed; USTAR / VSTAR are scratch in the reference.
        double hj2 = c.hj2;
        if (P.solid) hencky(P, c);
        if (P.solid) c.hj2 = hj2;
        stress(P, c);
        c.a = sound_speed(P, c);
#define APV(comp) ap[(long long)(comp)*cs + dst]
        for (int m = 0; m < P.M; ++m) {
            APV(P.A_ALPHA + m) = c.alpha[m];
            APV(P.A_ARHO + m) = c.arho[m];
            APV(P.A_RHOK + m) = c.rhok[m];
        }
        APV(P.A_RHO) = c.rho;
        for (int r = 0; r < 3; ++r) {
            APV(P.A_RHOU + r) = c.rhou[r];
            APV(P.A_VEL + r) = c.vel[r];
        }
        APV(P.A_E) = c.E;
        APV(P.A_P) = c.p;
        APV(P.A_A) = c.a;
        APV(P.A_USTAR) = 0.0;
        for (int qq = 0; qq < 9; ++qq) APV(P.A_SIGMA + qq) = c.sigma[qq];
        if (P.solid) {
            for (int qq = 0; qq < 9; ++qq) {
                APV(P.A_V + qq) = c.V[qq];
                APV(P.A_VSTAR + qq) = 0.0;
                APV(P.A_DEVH + qq) = c.devH[qq];
            }
            APV(P.A_HJ2) = c.hj2;
        }
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) {
                APV(P.A_EPS + m) = c.eps[m];
                APV(P.A_ARE + m) = c.are[m];
            }
        if (P.nmix) {
            APV(P.A_RMIX) = c.rm0;
            APV(P.A_RMIX + 1) = c.rm1;
            APV(P.A_LAM) = c.lam;
            APV(P.A_ARL) = c.arl;
        }
#undef APV
    }
}

__global__ void k_prim_to_state(DevParams P, Fp64Bufs b, int dom, const double* prim, double* X)
{
    const long long nt = b.ntot;
    const DevDomain D = b.doms[dom];
    const long long nd = (long long)D.n[0] * D.n[1] * D.n[2];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nd; t += (long long)gridDim.x * blockDim.x) {
        CellS c;
        int w = 0;
        for (int m = 0; m < P.M; ++m) c.alpha[m] = prim[(w++) * nd + t];
        for (int m = 0; m < P.M; ++m) c.rhok[m] = prim[(w++) * nd + t];
        for (int r = 0; r < 3; ++r) c.vel[r] = prim[(w++) * nd + t];
        c.p = prim[(w++) * nd + t];
        c.hj2 = 0.0;
        if (P.solid)
            for (int qq = 0; qq < 9; ++qq) c.V[qq] = prim[(w++) * nd + t];
        if (P.plastic)
            for (int m = 0; m < P.M; ++m) c.eps[m] = prim[(w++) * nd + t];
        if (P.nmix) {  // initialise.cpp:66-71
            c.lam = prim[(w++) * nd + t];
            c.rm0 = c.rhok[0];
            c.rm1 = c.rhok[0];
        }
        p2c(P, c);
        store_state(P, X, nt, D.off + t, c);
    }
}

// ---------------------------------------------------------------------------
// Global conservation sums in binary64: per cell alphaRho_k, rhoU and E times
// the cell volume, summed over the valid cells of every domain. The partition
// is fixed (kConsBlocks blocks of contiguous cell ranges, each thread a fixed
// stride, a fixed tree per block and over the blocks), so the result does
// not depend on the GPU or on scheduling: the same state gives the same bits.
// ---------------------------------------------------------------------------
static constexpr int kConsBlocks = kConsPartials;

__global__ void __launch_bounds__(kThreads) k_cons_partial(DevParams P, Fp64Bufs b, const double* X, double* part)
{
    const long long nt = b.ntot;
    const int nv = P.M + 4;
    const long long chunk = (nt + kConsBlocks - 1) / kConsBlocks;
    const long long g0 = blockIdx.x * chunk, g1 = min(nt, g0 + chunk);
    double acc[TJ_MAX_MAT + 4];
    for (int v = 0; v < TJ_MAX_MAT + 4; ++v) acc[v] = 0.0;
    int q = -1;
    long long qlo = 0, qhi = -1;  // cell range of domain q
    for (long long g = g0 + threadIdx.x; g < g1; g += kThreads) {
        if (g < qlo || g >= qhi) {
            q = find_dom(b.doms, b.ndom, g);
            qlo = b.doms[q].off;
            qhi = qlo + (long long)b.doms[q].n[0] * b.doms[q].n[1] * b.doms[q].n[2];
        }
        const DevDomain& D = b.doms[q];
        const double dv = D.dx[0] * (P.dim > 1 ? D.dx[1] : 1.0) * (P.dim > 2 ? D.dx[2] : 1.0);
        for (int m = 0; m < P.M; ++m) acc[m] += X[(P.S_ARHO + m) * nt + g] * dv;
        for (int r = 0; r < 3; ++r) acc[P.M + r] += X[(P.S_RHOU + r) * nt + g] * dv;
        acc[P.M + 3] += X[P.S_E * nt + g] * dv;
    }
    __shared__ double red[kThreads];
    for (int v = 0; v < nv; ++v) {
        red[threadIdx.x] = acc[v];
        __syncthreads();
        for (int h = kThreads / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[(long long)v * kConsBlocks + blockIdx.x] = red[0];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kConsBlocks) k_cons_final(int nv, const double* part, double* out)
{
    __shared__ double red[kConsBlocks];
    for (int v = 0; v < nv; ++v) {
        red[threadIdx.x] = part[(long long)v * kConsBlocks + threadIdx.x];
        __syncthreads();
        for (int h = kConsBlocks / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[v] = red[0];
        __syncthreads();
    }
}

// One AccessPattern component of one domain's valid cells (i fastest), with
// the derived components computed as in k_state_to_ap.
__global__ void k_state_component(DevParams P, Fp64Bufs b, int dom, const double* X, int comp, double* out)
{
    const long long nt = b.ntot;
    const DevDomain D = b.doms[dom];
    const long long nd = (long long)D.n[0] * D.n[1] * D.n[2];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nd; t += (long long)gridDim.x * blockDim.x) {
        CellS c;
        load_state(P, X, nt, D.off + t, nullptr, c);
        // the derived components in k_state_to_ap's order
        const double hj2 = c.hj2;
        if (P.solid) hencky(P, c);
        c.hj2 = hj2;
        stress(P, c);
        double v = 0.0;
        const auto in = [](int cmp, int first, int n) { return first >= 0 && cmp >= first && cmp < first + n; };
        if (in(comp, P.A_ALPHA, P.M)) v = c.alpha[comp - P.A_ALPHA];
        else if (in(comp, P.A_ARHO, P.M)) v = c.arho[comp - P.A_ARHO];
        else if (in(comp, P.A_RHOK, P.M)) v = c.rhok[comp - P.A_RHOK];
        else if (comp == P.A_RHO) v = c.rho;
        else if (in(comp, P.A_RHOU, 3)) v = c.rhou[comp - P.A_RHOU];
        else if (in(comp, P.A_VEL, 3)) v = c.vel[comp - P.A_VEL];
        else if (comp == P.A_E) v = c.E;
        else if (comp == P.A_P) v = c.p;
        else if (comp == P.A_A) v = sound_speed(P, c);
        else if (comp == P.A_USTAR || in(comp, P.A_VSTAR, 9)) v = 0.0;
        else if (in(comp, P.A_SIGMA, 9)) v = c.sigma[comp - P.A_SIGMA];
        else if (in(comp, P.A_DEVH, 9)) v = c.devH[comp - P.A_DEVH];
        else if (in(comp, P.A_V, 9)) v = c.V[comp - P.A_V];
        else if (comp == P.A_HJ2) v = c.hj2;
        else if (in(comp, P.A_EPS, P.M)) v = c.eps[comp - P.A_EPS];
        else if (in(comp, P.A_ARE, P.M)) v = c.are[comp - P.A_ARE];
        else if (comp == P.A_RMIX) v = c.rm0;
        else if (P.A_RMIX >= 0 && comp == P.A_RMIX + 1) v = c.rm1;
        else if (comp == P.A_LAM) v = c.lam;
        else if (comp == P.A_ARL) v = c.arl;
        out[t] = v;
    }
}

// ---------------------------------------------------------------------------
// Host launchers.
// ---------------------------------------------------------------------------
#define PROF_BEGIN(name) \
    if (pr) pr->begin(name, st)
#define PROF_END(name) \
    if (pr) pr->end(name, st)

int fp64_cfl(const DevParams& P, const Fp64Bufs& b, const double* X, cudaStream_t st, Prof* pr)
{
    return path_cfl_any(P, b, X, st, pr);
}

int fp64_dt_finalize(const DevParams& P, const Fp64Bufs& b, int clamp, cudaStream_t st)
{
    k_dt_finalize<<<1, 32, 0, st>>>(P, b.scal, clamp);
    return 1;
}

int fp64_stage(const DevParams& P, const Fp64Bufs& b, const double* X, double* Y, int finish, cudaStream_t st, Prof* pr)
{
    int n = 0;
    for (int d = 0; d < P.dim; ++d) n += path_dir_any(P, b, X, Y, d, d == 0, d == P.dim - 1, finish, st, pr);
    return n;
}

int fp64_step_end(const Fp64Bufs& b, cudaStream_t st)
{
    k_step_end<<<1, 32, 0, st>>>(b.scal);
    return 1;
}

int fp64_set_dt(const Fp64Bufs& b, double dt, cudaStream_t st)
{
    k_set_dt<<<1, 32, 0, st>>>(b.scal, dt);
    return 1;
}

int fp64_cell_op(const DevParams& P, const Fp64Bufs& b, double* X, const double* X2, int op, cudaStream_t st, double dt)
{
    k_cell_op<<<nblocks(b.ntot), kThreads, 0, st>>>(P, b, X, X2, op, dt);
    return 1;
}

int fp64_ap_to_state(const DevParams& P, const Fp64Bufs& b, int dom, const int* bx, const double* ap, int ld_i, int ld_j,
                     int ld_k, long long cs, int go, double* X, cudaStream_t st)
{
    (void)ld_k;
    int nx = bx[3] - bx[0] + 1, ny = bx[4] - bx[1] + 1, nz = bx[5] - bx[2] + 1;
    k_ap_to_state<<<nblocks((long long)nx * ny * nz), kThreads, 0, st>>>(P, b, dom, bx[0], bx[1], bx[2], nx, ny, nz, ap, ld_i,
                                                                         ld_j, cs, go, X);
    return 1;
}

int fp64_state_to_ap(const DevParams& P, const Fp64Bufs& b, int dom, const int* bx, const double* X, double* ap, int ld_i,
                     int ld_j, int ld_k, long long cs, int go, cudaStream_t st, long long t0, long long t1)
{
    (void)ld_k;
    int nx = bx[3] - bx[0] + 1, ny = bx[4] - bx[1] + 1, nz = bx[5] - bx[2] + 1;
    if (t1 < 0) t1 = (long long)nx * ny * nz;
    if (t1 <= t0) return 0;
    k_state_to_ap<<<nblocks(t1 - t0), kThreads, 0, st>>>(P, b, dom, bx[0], bx[1], bx[2], nx, ny, nz, X, ap, ld_i, ld_j,
                                                         cs, go, t0, t1);
    return 1;
}

int fp64_prim_to_state(const DevParams& P, const Fp64Bufs& b, int dom, const double* prim, double* X, cudaStream_t st)
{
    k_prim_to_state<<<nblocks(b.ntot), kThreads, 0, st>>>(P, b, dom, prim, X);
    return 1;
}

int fp64_conservation(const DevParams& P, const Fp64Bufs& b, const double* X, double* part, double* out, cudaStream_t st)
{
    k_cons_partial<<<kConsBlocks, kThreads, 0, st>>>(P, b, X, part);
    k_cons_final<<<1, kConsBlocks, 0, st>>>(P.M + 4, part, out);
    return 2;
}

int fp64_state_component(const DevParams& P, const Fp64Bufs& b, int dom, const double* X, int comp, double* out,
                         cudaStream_t st)
{
    k_state_component<<<nblocks(b.ntot), kThreads, 0, st>>>(P, b, dom, X, comp, out);
    return 1;
}

}  // namespace tj
