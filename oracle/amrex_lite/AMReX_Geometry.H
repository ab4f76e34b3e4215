// amrex_lite stand-in for AMReX_Geometry.H (oracle test infrastructure).
#include "amrex_lite.H"
