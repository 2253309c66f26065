// g2d_f32.cu -- FP32 step kernels with the genuinely-2D interface solver
// (HYDRO_SOLVER_G2D): the persistent TMA-staged kernel first (the default when
// nothing is tuned), then kernels that gather their tile.
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f32_g2d(std::vector<StepVariant<float>>& v)
{
    v.push_back(tma_variant<float, 32, 32, 512, 1, false, 2, HYDRO_SOLVER_G2D>());
    v.push_back(step_variant<float, 16, 32, 512, 2, false, HYDRO_SOLVER_G2D>());
    v.push_back(step_variant<float, 16, 16, 256, 4, false, HYDRO_SOLVER_G2D>());
    v.push_back(step_variant<float, 32, 32, 512, 1, false, HYDRO_SOLVER_G2D>());
}

}  // namespace hydro
