// Host builds of the FP64 device path's pow functions for the accuracy tests:
// the C library's method (libm_pow.cuh, the device default) and the correctly
// rounded double-double pow (hydro_pow.cuh, kept for comparison), each beside
// the host C library's pow for the same arguments.
#include <math.h>
#include "../../hydrocode-fusion_gb300/csrc/hydro_pow.cuh"
#include "../../hydrocode-fusion_gb300/csrc/libm_pow.cuh"

extern "C" void pow_pair(const double* x, const double* y, long long n, double* dd, double* libm)
{
    for (long long i = 0; i < n; ++i) {
        dd[i] = hydro::dd_pow(x[i], y[i]);
        libm[i] = pow(x[i], y[i]);
    }
}

extern "C" void lpow_pair(const double* x, const double* y, long long n, double* lp, double* libm)
{
    for (long long i = 0; i < n; ++i) {
        lp[i] = hydro::lpow(x[i], y[i]);
        libm[i] = pow(x[i], y[i]);
    }
}

// x^mu and x^nu from one logarithm (the wave curve and its slope) against two calls
extern "C" long long lpow_shared_log_mismatch(const double* x, long long n, double mu, double nu)
{
    long long bad = 0;
    for (long long i = 0; i < n; ++i) {
        hydro::LpowBase b;
        b.init(x[i]);
        bad += (b.pow_y(mu) != hydro::lpow(x[i], mu)) + (b.pow_y(nu) != hydro::lpow(x[i], nu));
    }
    return bad;
}
