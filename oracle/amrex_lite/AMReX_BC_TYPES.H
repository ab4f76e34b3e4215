// amrex_lite stand-in for AMReX_BC_TYPES.H (oracle test infrastructure).
#include "amrex_lite.H"
