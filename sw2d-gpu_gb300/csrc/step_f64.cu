// step_f64.cu -- FP64 instantiations.  Compiled with --fmad=false: every
// multiply and add rounds separately, as in the serial oracle and in the
// reference built without contraction, which makes the FP64 path
// bit-reproducible against them wherever no transcendental is involved.
#define SW2D_REAL double
#include "sw2d_launch_impl.cuh"

namespace sw2d {

// Fills this translation unit's tables of the deterministic log/exp (on the
// legacy stream, waited for: the handles' own streams do not order with it).
cudaError_t init_det_tables() {
    det_tables_kernel<<<1, 128>>>();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(0);
}

cudaError_t prepare_step(int th, int tw, double) {
    const cudaError_t e = init_det_tables();
    if (e != cudaSuccess) return e;
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
