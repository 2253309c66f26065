// f64_variants.cu -- FP64 (parity) step kernels; compiled with --fmad=false
// like the rest of the FP64 form.
#include "solver2d_impl.cuh"

namespace hydro {

void variants_f64(std::vector<StepVariant<double>>& v)
{
    v.push_back(step_variant<double, 16, 16, 256, 3>());
    v.push_back(step_variant<double, 8, 16, 128, 4>());
    v.push_back(tma_variant<double, 32, 16, 512, 1>());
}

}  // namespace hydro
