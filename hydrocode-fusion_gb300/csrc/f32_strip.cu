// f32_strip.cu -- FP32 strip step kernels (strip2d.cuh), plain and with the
// learned Newton starting pressure.
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f32_strip(std::vector<StepVariant<float>>& v, bool learned)
{
    if (learned) {
        v.push_back(strip_variant<4, 1, true>(32));
        v.push_back(strip_variant<8, 1, true>(32));
    } else {
        v.push_back(strip_variant<4, 1, false>(32));
        v.push_back(strip_variant<8, 1, false>(32));
    }
}

}  // namespace hydro
