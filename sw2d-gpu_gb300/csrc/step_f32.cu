// step_f32.cu -- FP32 instantiations (fast math: FMA contraction,
// approximate division, square root and power).  Accuracy is checked against
// the FP64 oracle with stated tolerances, not bit for bit.
#define SW2D_REAL float
#include "sw2d_launch_impl.cuh"
#include "sw2d_stream.cuh"

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

int stream_out_cols() { return kStreamOut; }

cudaError_t prepare_stream_step() {
    return cudaFuncSetAttribute(stream_step_kernel<kStreamWarps>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxL1);
}

cudaError_t launch_stream_step(int nblocks, int tiles_w, int strip_h, int units, const GridDesc &G,
                               const ForcingDesc &F, const StateBufs<float> &S, const Thr<float> &T, Clock *clk,
                               const Control *ctl, int slot, cudaStream_t st) {
    StreamShape sh;
    sh.tiles_w = tiles_w;
    sh.strip_h = strip_h;
    sh.units = units;
    sh.pad = 0;
    stream_step_kernel<kStreamWarps><<<nblocks, kStreamWarps * 32, 0, st>>>(G, F, S, T, clk, ctl, slot, sh);
    return cudaGetLastError();
}

}  // namespace sw2d
