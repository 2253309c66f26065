// TEST INFRASTRUCTURE ONLY: exposes the FP64 device path's pow (host build of
// hydrocode-fusion_gb300/csrc/libm_pow.cuh, the C library's table-driven
// method) under a C name, so oracle/Makefile can build a twin of the oracle
// whose pow() is the device's.
#include <math.h>

#include "../hydrocode-fusion_gb300/csrc/libm_pow.cuh"

extern "C" double hydro_lpow(double x, double y) { return hydro::lpow(x, y); }
