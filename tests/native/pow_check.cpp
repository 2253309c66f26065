// Host build of the device double-double pow (hydro_pow.cuh) for the accuracy
// test: returns both it and the C library's pow for the given arguments.
#include <math.h>
#include "../../hydrocode-fusion_gb300/csrc/hydro_pow.cuh"

extern "C" void pow_pair(const double* x, const double* y, long long n, double* dd, double* libm)
{
    for (long long i = 0; i < n; ++i) {
        dd[i] = hydro::dd_pow(x[i], y[i]);
        libm[i] = pow(x[i], y[i]);
    }
}
