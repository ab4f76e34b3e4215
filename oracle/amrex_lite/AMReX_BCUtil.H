// amrex_lite stand-in for AMReX_BCUtil.H (oracle test infrastructure).
#include "amrex_lite.H"
