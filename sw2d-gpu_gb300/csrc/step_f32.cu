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

// Shared-memory share of the L1/shared split for the streaming kernel, in
// percent.  Each CTA needs only a few KB (source slots and the reduction, plus
// the 1 KB the system reserves), but asking for the largest L1 left room for
// just 2-3 CTAs per SM and capped the occupancy of the smaller-CTA builds.
constexpr int kStreamCarveoutPercent = 25;

// Builds of the streaming kernel the autotuner chooses from: (id, warps per
// CTA, minimum resident CTAs per SM -- which sets the register budget: 20
// warps per SM fit 96 registers, 16 fit 128, 24 fit 80 --, unrolling of the
// row loop).  Build 0 is the default.
#define SW2D_STREAM_VARIANTS(X) \
    X(0, 2, 10, 2) X(1, 2, 10, 1) X(2, 4, 5, 2) X(3, 8, 2, 1) X(4, 8, 2, 2) X(5, 12, 2, 1)

int stream_variants() { return 6; }

int stream_warps(int variant) {
#define SW2D_W(id, nw, mb, un) \
    if (variant == id) return nw;
    SW2D_STREAM_VARIANTS(SW2D_W)
#undef SW2D_W
    return 4;
}

cudaError_t prepare_stream_step(int variant) {
#define SW2D_P(id, nw, mb, un)                                                                            \
    if (variant == id) {                                                                               \
        const void *k[4] = {(const void *)stream_step_kernel<nw, mb, un, false, false>,                \
                            (const void *)stream_step_kernel<nw, mb, un, false, true>,                 \
                            (const void *)stream_step_kernel<nw, mb, un, true, false>,                 \
                            (const void *)stream_step_kernel<nw, mb, un, true, true>};                 \
        for (const void *f : k) {                                                                      \
            cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout,   \
                                                 kStreamCarveoutPercent);                             \
            if (e != cudaSuccess) return e;                                                            \
        }                                                                                              \
        return cudaSuccess;                                                                            \
    }
    SW2D_STREAM_VARIANTS(SW2D_P)
#undef SW2D_P
    return cudaErrorInvalidValue;
}

const char *stream_variant_name(int variant) {
#define SW2D_N(id, nw, mb, un) \
    if (variant == id) return "stream_step_kernel<" #nw "," #mb "," #un ">";
    SW2D_STREAM_VARIANTS(SW2D_N)
#undef SW2D_N
    return "stream_step_kernel<?>";
}

int stream_ctas_per_sm(int variant) {
    int n = 0;
#define SW2D_O(id, nw, mb, un)                                                                           \
    if (variant == id &&                                                                                 \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stream_step_kernel<nw, mb, un, false, false>, nw * 32, 0) != \
            cudaSuccess)                                                                                 \
        n = 0;
    SW2D_STREAM_VARIANTS(SW2D_O)
#undef SW2D_O
    return n;
}

cudaError_t launch_stream_step(int variant, int nblocks, int tiles_w, int strip_h, int units, const GridDesc &G,
                               const ForcingDesc &F, const StateBufs<float> &S, const Thr<float> &T, Clock *clk,
                               const Control *ctl, int slot, cudaStream_t st) {
    StreamShape sh;
    sh.tiles_w = tiles_w;
    sh.strip_h = strip_h;
    sh.units = units;
    sh.pad = 0;
    // the general build carries the moving storm and the point sources
    const bool gen = F.rain_kind == RAIN_STORM || G.n_src > 0;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(nblocks);
    lc.dynamicSmemBytes = 0;
    lc.stream = st;
    lc.attrs = attr;
    lc.numAttrs = 1;
#define SW2D_L(id, nw, mb, un)                                                                             \
    if (variant == id) {                                                                                 \
        lc.blockDim = dim3(nw * 32);                                                                     \
        if (S.rainw && gen)                                                                              \
            return cudaLaunchKernelEx(&lc, stream_step_kernel<nw, mb, un, true, true>, G, F, S, T, clk, ctl, slot, sh);   \
        else if (S.rainw)                                                                                \
            return cudaLaunchKernelEx(&lc, stream_step_kernel<nw, mb, un, true, false>, G, F, S, T, clk, ctl, slot, sh);  \
        else if (gen)                                                                                    \
            return cudaLaunchKernelEx(&lc, stream_step_kernel<nw, mb, un, false, true>, G, F, S, T, clk, ctl, slot, sh);  \
        else                                                                                             \
            return cudaLaunchKernelEx(&lc, stream_step_kernel<nw, mb, un, false, false>, G, F, S, T, clk, ctl, slot, sh); \
    }
    SW2D_STREAM_VARIANTS(SW2D_L)
#undef SW2D_L
    return cudaErrorInvalidValue;
}

}  // namespace sw2d
