// g2d_f64.cu -- FP64 (parity) step kernels with the genuinely-2D interface
// solver (HYDRO_SOLVER_G2D); compiled with --fmad=false like the rest of the
// FP64 form.
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f64_g2d(std::vector<StepVariant<double>>& v)
{
    v.push_back(step_variant<double, 16, 16, 256, 3, false, HYDRO_SOLVER_G2D>());
    v.push_back(step_variant<double, 8, 16, 128, 4, false, HYDRO_SOLVER_G2D>());
}

}  // namespace hydro
