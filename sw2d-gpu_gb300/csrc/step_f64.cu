// step_f64.cu -- FP64 instantiations.  Compiled with --fmad=false: every
// multiply and add rounds separately, as in the serial oracle and in the
// reference built without contraction, which makes the FP64 path
// bit-reproducible against them wherever no transcendental is involved.
#define SW2D_REAL double
#include "sw2d_launch_impl.cuh"

namespace sw2d {

cudaError_t prepare_step(int th, int tw, double) {
    if (th == 16 && tw == 32) return detail::step_prepare<double, 16, 32, 256>();
    if (th == 8 && tw == 32) return detail::step_prepare<double, 8, 32, 128>();
    return cudaErrorInvalidValue;
}

cudaError_t launch_step(int th, int tw, int nblocks, const GridDesc &G, const ForcingDesc &F,
                        const StateBufs<double> &S, const Thr<double> &T, Clock *clk, const Control *ctl, int slot,
                        cudaStream_t st) {
    if (th == 16 && tw == 32) return detail::step_launch<double, 16, 32, 256>(nblocks, G, F, S, T, clk, ctl, slot, st);
    if (th == 8 && tw == 32) return detail::step_launch<double, 8, 32, 128>(nblocks, G, F, S, T, clk, ctl, slot, st);
    return cudaErrorInvalidValue;
}

}  // namespace sw2d
