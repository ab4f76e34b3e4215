// amrex_lite stand-in for AMReX_MultiFab.H (oracle test infrastructure).
#include "amrex_lite.H"
