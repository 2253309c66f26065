// f32_strip.cu -- FP32 strip step kernels (strip2d.cuh), plain and with the
// learned Newton starting pressure.  Listed first: index 0 is the default when
// nothing is tuned (the scheme entry points), and these are the fastest FP32
// step kernels on the grids measured (2048^2, 4096^2).
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f32_strip(std::vector<StepVariant<float>>& v, bool learned)
{
    // 4 warps per CTA; units of 16 or 32 rows; half of the L1/shared storage
    // left as L1 for the kernel's register spills
    if (learned) {
        v.push_back(strip_variant<4, 1, true>(16, 50));
        v.push_back(strip_variant<4, 1, true>(32, 50));
    } else {
        v.push_back(strip_variant<4, 1, false>(16, 50));
        v.push_back(strip_variant<4, 1, false>(32, 50));
    }
}

}  // namespace hydro
