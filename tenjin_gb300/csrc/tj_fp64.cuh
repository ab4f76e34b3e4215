// FP64 reference-faithful kernels of the per-timestep update.
#pragma once

#include "tj_types.h"

namespace tj {

template <typename R>
struct PathBufs {
    R *A, *B, *C;        // state: U^n (and result), stage-1 output, stage-2 partial
    R *UL, *UR;          // reconstructed face states, one per cell
    R* FX;               // face fluxes of the current direction
    R *ulstar, *urstar;  // THINC scratch (alpha of the reference's ULStar / URStar)
    R* gstar[3];         // ULStar ghost alpha at box hi+1 faces, per direction
    int* cell_box;            // domain-local box index of each cell
    int* boxes;               // 6 ints per box, all domains
    DevDomain* doms;
    DevScalars* scal;
    long long ntot, nftot[3];
    int ndom;
    // optional record of the reconstruction (for the adjoint's recompute):
    // alpha of UL and UR after the BVD choice, before cleanUpAlpha, at
    // rec[((d * 2 + side) * M + m) * ntot + g], and per cell and direction
    // 2 bits per material at rec_code[d * ntot + g]: 0 MUSCL, 1 the cell's
    // own THINC candidate, 2 a value of the THINC scratch
    R* rec = nullptr;
    int* rec_code = nullptr;
};
using Fp64Bufs = PathBufs<double>;

// The binary32 parameter block of a binary64 one (tj_fp32.cu).
DevParams32 make_params32(const DevParams& P);

// Launch helpers (tj_fp64.cu). Each returns the number of kernel launches.
int fp64_cfl(const DevParams& P, const Fp64Bufs& b, const double* X, cudaStream_t st, Prof* pr = nullptr);
int fp64_dt_finalize(const DevParams& P, const Fp64Bufs& b, int use_clamp, cudaStream_t st);
int fp64_stage(const DevParams& P, const Fp64Bufs& b, const double* X, double* Y, int finish, cudaStream_t st,
               Prof* pr = nullptr);
int fp64_step_end(const Fp64Bufs& b, cudaStream_t st);
int fp64_set_dt(const Fp64Bufs& b, double dt, cudaStream_t st);

// Whole-array operators of the C ABI.
enum CellOp { OP_C2P = 0, OP_P2C = 1, OP_CLEAN_ALPHA = 2, OP_CLEAN_V = 3, OP_PLASTIC = 4, OP_NAN = 5, OP_AVERAGE = 6,
              OP_RADIAL = 7, OP_REACTIVE = 8 };
int fp64_cell_op(const DevParams& P, const Fp64Bufs& b, double* X, const double* X2, int op, cudaStream_t st,
                 double dt = 0.0);

// Layout conversion: AccessPattern blocks (valid cells of one box of one
// domain, ncomp x box cells, i fastest) <-> carried state.
int fp64_ap_to_state(const DevParams& P, const Fp64Bufs& b, int dom, const int* box_lohi, const double* ap, int ld_i,
                     int ld_j, int ld_k, long long cstride, int ghost_off, double* X, cudaStream_t st);
// Cells [t0, t1) of the box (box-linear index, i fastest); t1 < 0: all.
int fp64_state_to_ap(const DevParams& P, const Fp64Bufs& b, int dom, const int* box_lohi, const double* X, double* ap,
                     int ld_i, int ld_j, int ld_k, long long cstride, int ghost_off, cudaStream_t st,
                     long long t0 = 0, long long t1 = -1);
int fp64_prim_to_state(const DevParams& P, const Fp64Bufs& b, int dom, const double* prim, double* X, cudaStream_t st);

// Deterministic binary64 sums over all valid cells of alphaRho_k (M), rhoU
// (3) and E, each times the cell volume: out[M + 4] (device), part: scratch of
// kConsPartials * (M + 4) doubles.
constexpr int kConsPartials = 256;
int fp64_conservation(const DevParams& P, const Fp64Bufs& b, const double* X, double* part, double* out, cudaStream_t st);
// One AccessPattern component of domain dom (valid cells, i fastest) into
// out (device).
int fp64_state_component(const DevParams& P, const Fp64Bufs& b, int dom, const double* X, int comp, double* out,
                         cudaStream_t st);

}  // namespace tj
