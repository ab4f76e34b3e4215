// amrex_lite stand-in for AMReX_Print.H (oracle test infrastructure).
#include "amrex_lite.H"
