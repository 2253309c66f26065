// solver2d_f32.cu -- FP32 instantiation of the 2D solver (FP32 state and
// fluxes; the exact solver falls back to FP64 near vacuum / on non-convergence).
#include "solver2d_impl.cuh"

namespace hydro {

Solver2DBase* make_solver2d_f32(int m, int n, int learned, int rs)
{
    Solver2D<float>* s = new Solver2D<float>();
    if (s->init(m, n, learned ? HYDRO_FORM_FP32_LEARNED : HYDRO_FORM_FP32, rs)) {
        delete s;
        return nullptr;
    }
    return s;
}

}  // namespace hydro
