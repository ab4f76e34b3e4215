// amrex_lite stand-in for AMReX_BCRec.H (oracle test infrastructure).
#include "amrex_lite.H"
