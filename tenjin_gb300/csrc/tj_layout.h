// Component layouts of the device arrays and of the reference's
// AccessPattern (accesspattern.cpp:44-79), derived from the parameters. Shared
// by the context-based entry points and the allocation-free ones, so that both
// read a caller's state at the same offsets.
#pragma once

#include <cstring>

#include "tj_types.h"

namespace tj {

inline void make_layouts(const tj_params& p, DevParams& P)
{
    std::memset(&P, 0, sizeof P);
    P.dim = p.dim;
    P.M = p.n_materials;
    P.solid = p.SOLID;
    P.thinc = p.THINC;
    P.plastic = p.PLASTIC;
    P.muscl = p.MUSCL;
    P.fused64 = p.precision == TJ_PRECISION_FUSED64;
    P.radial = p.RADIAL ? 1 : 0;
    P.nmix = p.n_mixtures;
    P.reactive = p.REACTIVE ? 1 : 0;
    P.S_ELO = -1;
    for (int d = 0; d < 3; ++d) { P.lo_bc[d] = p.lo_bc[d]; P.hi_bc[d] = p.hi_bc[d]; }
    P.cfl = p.CFL;
    P.beta = p.THINCbeta;
    for (int m = 0; m < P.M; ++m) {
        P.phase[m] = p.materials[m].phase;
        P.eos[m] = p.materials[m].eos;
        for (int q = 0; q < TJ_MAX_EOS_PARAMS; ++q) P.prm[m][q] = q < p.materials[m].nparams ? p.materials[m].params[q] : 0.0;
        P.yield[m] = p.materials[m].yield_stress;
        if (P.phase[m] == TJ_PHASE_SOLID) P.any_solid = 1;
    }
    int M = P.M, n = 0;
    P.S_ALPHA = n; n += M;
    P.S_ARHO = n; n += M;
    P.S_RHOK = n; n += M;
    P.S_RHO = n++;
    P.S_RHOU = n; n += 3;
    P.S_VEL = n; n += 3;
    P.S_E = n++;
    P.S_P = n++;
    P.S_V = P.S_HJ2 = P.S_EPS = P.S_ARE = -1;
    if (P.solid) { P.S_V = n; n += 9; P.S_HJ2 = n++; }
    if (P.plastic) { P.S_EPS = n; n += M; P.S_ARE = n; n += M; }
    P.S_RMIX = P.S_LAM = P.S_ARL = -1;
    if (P.nmix) { P.S_RMIX = n; n += 2; P.S_LAM = n++; P.S_ARL = n++; }
    P.NS = n;
    n = 0;
    P.F_ALPHA = n; n += M;
    P.F_ARHO = n; n += M;
    P.F_RHO = n++;
    P.F_RHOU = n; n += 3;
    P.F_VEL = n; n += 3;
    P.F_E = n++;
    P.F_P = n++;
    P.F_A = n++;
    P.F_SIGMA = P.F_V = P.F_ARE = -1;
    if (P.solid) { P.F_SIGMA = n; n += 9; P.F_V = n; n += 9; }
    if (P.plastic) { P.F_ARE = n; n += M; }
    P.F_ARL = P.nmix ? n++ : -1;
    P.NF = n;
    n = 0;
    P.X_ALPHA = n; n += M;
    P.X_ARHO = n; n += M;
    P.X_RHOU = n; n += 3;
    P.X_E = n++;
    P.X_V = P.X_ARE = -1;
    if (P.solid) { P.X_V = n; n += 9; }
    if (P.plastic) { P.X_ARE = n; n += M; }
    P.X_ARL = P.nmix ? n++ : -1;
    P.X_SSTAR = n++;
    P.X_VSTAR = -1;
    if (P.solid) { P.X_VSTAR = n; n += 3; }
    P.NX = n;
    // AccessPattern (accesspattern.cpp:44-79)
    n = 0;
    P.A_ALPHA = n; n += M;
    P.A_ARHO = n; n += M;
    P.A_RHOK = n; n += M;
    P.A_RHO = n++;
    P.A_RHOU = n; n += 3;
    P.A_VEL = n; n += 3;
    P.A_E = n++;
    P.A_P = n++;
    P.A_A = n++;
    P.A_USTAR = n++;
    P.A_SIGMA = n; n += 9;
    P.A_RMIX = P.A_LAM = P.A_ARL = -1;
    if (P.nmix) { P.A_RMIX = n; n += 2; P.A_LAM = n++; P.A_ARL = n++; }
    P.A_V = P.A_VSTAR = P.A_DEVH = P.A_HJ2 = P.A_EPS = P.A_ARE = -1;
    if (P.solid) {
        P.A_V = n; n += 9;
        P.A_VSTAR = n; n += 9;
        P.A_DEVH = n; n += 9;
        P.A_HJ2 = n++;
        if (P.plastic) { P.A_EPS = n; n += M; P.A_ARE = n; n += M; }
    }
    P.NCOMP = n;
}

}  // namespace tj
