// amrex_lite stand-in for AMReX_PlotFileUtil.H (oracle test infrastructure).
#include "amrex_lite.H"
