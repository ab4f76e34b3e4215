// amrex_lite stand-in for AMReX_iMultiFab.H (oracle test infrastructure).
#include "amrex_lite.H"
