// amrex_lite stand-in for AMReX_Array.H (oracle test infrastructure).
#include "amrex_lite.H"
