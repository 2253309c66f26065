// f32_strip.cu -- FP32 strip step kernels (strip2d.cuh), plain and with the
// learned Newton starting pressure.  Listed first: index 0 is the default when
// nothing is tuned (the scheme entry points), and these are the fastest FP32
// step kernels on the grids measured (2048^2, 4096^2).
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f32_strip(std::vector<StepVariant<float>>& v, bool learned)
{
    // 4 warps per CTA; units of 16 or 32 rows; the L1/shared split: the
    // smallest shared-memory configuration that holds two CTAs (64 KB; 100 KB
    // with the network image in shared memory) and the rest as L1, or half of
    // the storage as L1.  Learned form: the network image read through L1 or
    // staged in shared memory; the network on queue flushes of at least 16
    // faces or only on full warps of 32.  The first of each list is the
    // fastest at 4096^2 (the default when nothing is tuned).
    if (learned) {
        v.push_back(strip_variant<4, 1, true>(16, 28, 32, 1));
        v.push_back(strip_variant<4, 1, true>(16, 28, 16, 1));
        v.push_back(strip_variant<4, 1, true>(32, 28, 32, 1));
        v.push_back(strip_variant<4, 1, true>(16, 43, 32));
        v.push_back(strip_variant<4, 1, true>(16, 43));
        v.push_back(strip_variant<4, 1, true>(16, 50));
        v.push_back(strip_variant<4, 1, true>(32, 50));
    } else {
        v.push_back(strip_variant<4, 1, false>(16, 28));
        v.push_back(strip_variant<4, 1, false>(32, 28));
        v.push_back(strip_variant<4, 1, false>(16, 50));
        v.push_back(strip_variant<4, 1, false>(32, 50));
    }
}

}  // namespace hydro
