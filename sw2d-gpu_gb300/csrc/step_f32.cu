// step_f32.cu -- FP32 instantiations (fast math: FMA contraction,
// approximate division, square root and power).  Accuracy is checked against
// the FP64 oracle with stated tolerances, not bit for bit.
#define SW2D_REAL float
#include "sw2d_launch_impl.cuh"

namespace sw2d {

cudaError_t prepare_step(int th, int tw, float) {
    if (th == 16 && tw == 32) return detail::step_prepare<float, 16, 32, 256>();
    if (th == 32 && tw == 32) return detail::step_prepare<float, 32, 32, 256>();
    if (th == 16 && tw == 64) return detail::step_prepare<float, 16, 64, 256>();
    return cudaErrorInvalidValue;
}

cudaError_t launch_step(int th, int tw, int nblocks, const GridDesc &G, const ForcingDesc &F,
                        const StateBufs<float> &S, const Thr<float> &T, Clock *clk, const Control *ctl, int slot,
                        cudaStream_t st) {
    if (th == 16 && tw == 32) return detail::step_launch<float, 16, 32, 256>(nblocks, G, F, S, T, clk, ctl, slot, st);
    if (th == 32 && tw == 32) return detail::step_launch<float, 32, 32, 256>(nblocks, G, F, S, T, clk, ctl, slot, st);
    if (th == 16 && tw == 64) return detail::step_launch<float, 16, 64, 256>(nblocks, G, F, S, T, clk, ctl, slot, st);
    return cudaErrorInvalidValue;
}

}  // namespace sw2d
