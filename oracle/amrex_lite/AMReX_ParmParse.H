// amrex_lite stand-in for AMReX_ParmParse.H (oracle test infrastructure).
#include "amrex_lite.H"
