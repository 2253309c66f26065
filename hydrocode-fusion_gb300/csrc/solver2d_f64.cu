// solver2d_f64.cu -- FP64 (parity) instantiation of the 2D solver.
// Compiled with --fmad=false: no multiply-add contraction, IEEE division and
// square root, so every operation rounds exactly as the reference's C code,
// pow() included (libm_pow.cuh follows the C library's own method).
#include "solver2d_impl.cuh"

namespace hydro {

Solver2DBase* make_solver2d_f64(int m, int n, int rs)
{
    Solver2D<double>* s = new Solver2D<double>();
    if (s->init(m, n, HYDRO_FORM_FP64, rs)) {
        delete s;
        return nullptr;
    }
    return s;
}

}  // namespace hydro

// The FP64 form's uniform-pair threshold (the host side of the kernels' test).
extern "C" double hydro_uniform_dist2_max(double eps) { return hydro::uniform_dist2_max(eps); }
