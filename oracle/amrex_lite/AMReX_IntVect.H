// amrex_lite stand-in for AMReX_IntVect.H (oracle test infrastructure).
#include "amrex_lite.H"
