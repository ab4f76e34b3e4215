// Empty stand-in for libconfig++ (test infrastructure only). The reference
// includes it from simulationheader.h:14; only initialise.cpp uses it, and the
// oracle harness replaces initialise.cpp.
