// Internal types shared by the host C-ABI layer and the kernels.
#pragma once

#include "tenjin_gpu.h"

#define TJ_MAX_MAT TJ_MAX_MATERIALS

namespace tj {

// Device copy of the solver parameters plus the layouts of the device
// arrays (component offsets). Passed to kernels by value.
struct DevParams {
    using real = double;
    int dim, M, solid, thinc, plastic, muscl, any_solid;
    int fused64;  // fused kernels in binary64 (TJ_PRECISION_FUSED64)
    int radial;   // RADIAL: geometric source term after the plastic update
    int nmix;     // numberOfMixtures (0 or 1; material 0 holds the MixtureEOS)
    int reactive; // REACTIVE: reactiveUpdate after advance
    int lo_bc[3], hi_bc[3];
    double cfl, beta;
    int phase[TJ_MAX_MAT], eos[TJ_MAX_MAT];
    double prm[TJ_MAX_MAT][TJ_MAX_EOS_PARAMS];
    double yield[TJ_MAX_MAT];
    // carried state (one SoA block of ntot cells per word)
    int S_ALPHA, S_ARHO, S_RHOK, S_RHO, S_RHOU, S_VEL, S_E, S_P, S_V, S_HJ2, S_EPS, S_ARE, NS;
    int S_RMIX, S_LAM, S_ARL;  // mixture: rhomix (2), lambda, alphaRhoLambda; -1 without
    // reconstructed face state (UL / UR)
    int F_ALPHA, F_ARHO, F_RHO, F_RHOU, F_VEL, F_E, F_P, F_A, F_SIGMA, F_V, F_ARE, NF;
    int F_ARL;
    // face flux
    int X_ALPHA, X_ARHO, X_RHOU, X_E, X_SSTAR, X_V, X_VSTAR, X_ARE, NX;
    int X_ARL;
    // AccessPattern (reference component order)
    int A_ALPHA, A_ARHO, A_RHOK, A_RHO, A_RHOU, A_VEL, A_E, A_P, A_A, A_USTAR, A_SIGMA, A_V, A_VSTAR, A_DEVH, A_HJ2,
        A_EPS, A_ARE, NCOMP;
    int A_RMIX, A_LAM, A_ARL;
    int S_ELO;  // binary32 state only (the low word of the energy); -1 here
};

// The same block for the binary32 instance of the per-direction kernels: the
// EOS parameters in binary32, the carried state one word longer (S_ELO), and
// the binary64 block for the pressure closure and the yield projection.
struct DevParams32 {
    using real = float;
    int dim, M, solid, thinc, plastic, muscl, any_solid;
    int fused64;
    int radial;
    int nmix, reactive;
    int lo_bc[3], hi_bc[3];
    float cfl, beta;
    int phase[TJ_MAX_MAT], eos[TJ_MAX_MAT];
    float prm[TJ_MAX_MAT][TJ_MAX_EOS_PARAMS];
    float yield[TJ_MAX_MAT];
    int S_ALPHA, S_ARHO, S_RHOK, S_RHO, S_RHOU, S_VEL, S_E, S_P, S_V, S_HJ2, S_EPS, S_ARE, NS;
    int S_RMIX, S_LAM, S_ARL;
    int F_ALPHA, F_ARHO, F_RHO, F_RHOU, F_VEL, F_E, F_P, F_A, F_SIGMA, F_V, F_ARE, NF;
    int F_ARL;
    int X_ALPHA, X_ARHO, X_RHOU, X_E, X_SSTAR, X_V, X_VSTAR, X_ARE, NX;
    int X_ARL;
    int S_ELO;
    DevParams d;
    // binary64 reciprocals for the closure of the binary32 cells:
    // 1 / (prm[m][0] - 1) and 0.5 / prm[m][4]
    double rG[TJ_MAX_MAT], rR0h[TJ_MAX_MAT];
};

// A parameter block whose material count is a compile-time constant: the
// static member M hides the base's runtime M, so that the per-material loops
// of the kernels unroll and their per-material arrays stay in registers.
template <class Base, int MC>
struct WithM : Base {
    static constexpr int M = MC;
    WithM() = default;
    explicit WithM(const Base& b) : Base(b) {}
};

// One independent domain: valid cells [0,n) per axis, stored contiguously
// from cell offset `off` (i fastest) in every state block.
struct DevDomain {
    int n[3];
    double dx[3];
    long long off;        // first cell in the concatenated cell space
    long long foff[3];    // first face of direction d in the face space of d
    int box_off, nbox;    // range in the box table
};

// Scalars kept on the device for graph-captured time stepping.
struct DevScalars {
    double t, dt, t_end, dtmin_raw;
    unsigned long long dtmin_bits;  // atomicMin over positive doubles as bits
    int n, status, done, nan_flag;
};

// Launch-timing hook: begin/end bracket one kernel launch on a stream.
struct Prof {
    virtual void begin(const char* kernel, void* stream) = 0;
    virtual void end(const char* kernel, void* stream) = 0;
    virtual ~Prof() {}
};

}  // namespace tj
