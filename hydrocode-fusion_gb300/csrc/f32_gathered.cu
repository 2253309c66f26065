// f32_gathered.cu -- FP32 step kernels that gather their tile (one CTA per tile).
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f32_gathered(std::vector<StepVariant<float>>& v)
{
    v.push_back(step_variant<float, 16, 16, 256, 4>());
    v.push_back(step_variant<float, 16, 32, 512, 2>());
    v.push_back(step_variant<float, 32, 32, 512, 1>());
}

}  // namespace hydro
