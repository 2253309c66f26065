// f32_learned.cu -- FP32 step kernels with the learned Newton starting pressure.
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f32_learned(std::vector<StepVariant<float>>& v)
{
    // the TMA-staged kernels before the gathered ones
    v.push_back(tma_variant<float, 32, 32, 512, 1, true>());
    v.push_back(tma_variant<float, 32, 32, 384, 1, true>());
    v.push_back(tma_variant<float, 16, 32, 256, 2, true, 1>());
    v.push_back(step_variant<float, 32, 32, 512, 1, true>());
    v.push_back(step_variant<float, 16, 32, 512, 2, true>());
}

}  // namespace hydro
