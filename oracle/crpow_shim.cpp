// TEST INFRASTRUCTURE ONLY: exposes the FP64 device path's double-double pow
// (host build of hydrocode-fusion_gb300/csrc/hydro_pow.cuh) under a C name, so
// oracle/Makefile can build a twin of the oracle whose pow() is correctly rounded.
#include <math.h>

#include "../hydrocode-fusion_gb300/csrc/hydro_pow.cuh"

extern "C" double hydro_crpow(double x, double y) { return hydro::dd_pow(x, y); }
