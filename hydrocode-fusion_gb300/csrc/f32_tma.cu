// f32_tma.cu -- FP32 persistent TMA-staged step kernels.
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f32_tma(std::vector<StepVariant<float>>& v)
{
    v.push_back(tma_variant<float, 32, 32, 512, 1>());
    v.push_back(tma_variant<float, 32, 32, 384, 1>());
    v.push_back(tma_variant<float, 16, 32, 256, 2, false, 1>());
}

}  // namespace hydro
