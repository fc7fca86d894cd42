// step_f32.cu -- FP32 instantiations (fast math: FMA contraction,
// approximate division, square root and power).  Accuracy is checked against
// the FP64 oracle with stated tolerances, not bit for bit.
#define SW2D_REAL float
#include "sw2d_launch_impl.cuh"
#include "sw2d_pipe.cuh"
#include "sw2d_stream.cuh"

#include <cstring>
#include <numeric>

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

namespace {

// The launch shape: ceil(rows / strip_h) strips, split evenly or with the
// heights skewed (strip_rows); for the pipelined launches the units go to
// warps in a scattered order (a multiplier near 0.618 units, coprime with
// units).
StreamShape stream_shape(int rows, int tiles_w, int strip_h, int units, bool scatter, int skew) {
    StreamShape sh;
    std::memset(&sh, 0, sizeof(sh));
    sh.tiles_w = tiles_w;
    sh.strips = (rows + strip_h - 1) / strip_h;
    sh.units = units;
    sh.perm = 1;
    sh.skew = skew;
    if (scatter && units > 2) {
        int p = (int)(units * 0.6180339887498949);
        if (p < 1) p = 1;
        while (std::gcd(p, units) != 1) p++;
        sh.perm = p;
    }
    return sh;
}

}  // namespace

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

// Build 6: the shape of build 0 with its rows staged in shared memory by TMA
// (stream_step_tma_kernel), for uniform forcing; the other forcing forms run
// build 0 (the same arithmetic, the same bits).
constexpr int kTmaVariant = 6;
constexpr size_t kTmaSmem = (size_t)2 * kTmaStages * kTmaStageBytes;

int stream_variants() { return 7; }

int stream_warps(int variant) {
    if (variant == kTmaVariant) return 2;
#define SW2D_W(id, nw, mb, un) \
    if (variant == id) return nw;
    SW2D_STREAM_VARIANTS(SW2D_W)
#undef SW2D_W
    return 4;
}

cudaError_t prepare_stream_step(int variant) {
    if (variant == kTmaVariant) {
        cudaError_t e = cudaFuncSetAttribute(stream_step_tma_kernel<2, 10, 2>,
                                             cudaFuncAttributePreferredSharedMemoryCarveout,
                                             (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(stream_step_tma_kernel<2, 10, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kTmaSmem);
        if (e != cudaSuccess) return e;
        variant = 0;  // the build the other forcing forms run
    }
#define SW2D_P(id, nw, mb, un)                                                                            \
    if (variant == id) {                                                                               \
        const void *k[4] = {(const void *)stream_step_kernel<nw, mb, un, false, false>,                \
                            (const void *)stream_step_kernel<nw, mb, un, false, true>,                 \
                            (const void *)stream_step_kernel<nw, mb, un, true, false>,                 \
                            (const void *)stream_step_kernel<nw, mb, un, true, true>};                 \
        const void *p[4] = {(const void *)stream_pipe_kernel<nw, mb, un, false, false>,                \
                            (const void *)stream_pipe_kernel<nw, mb, un, false, true>,                 \
                            (const void *)stream_pipe_kernel<nw, mb, un, true, false>,                 \
                            (const void *)stream_pipe_kernel<nw, mb, un, true, true>};                 \
        for (int i = 0; i < 8; i++) {                                                                  \
            cudaError_t e = cudaFuncSetAttribute(i < 4 ? k[i] : p[i - 4],                              \
                                                 cudaFuncAttributePreferredSharedMemoryCarveout,       \
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
    if (variant == kTmaVariant) return "stream_step_tma_kernel<2,10,2>";
#define SW2D_N(id, nw, mb, un) \
    if (variant == id) return "stream_step_kernel<" #nw "," #mb "," #un ">";
    SW2D_STREAM_VARIANTS(SW2D_N)
#undef SW2D_N
    return "stream_step_kernel<?>";
}

int stream_ctas_per_sm(int variant) {
    int n = 0;
    if (variant == kTmaVariant)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stream_step_tma_kernel<2, 10, 2>, 64, kTmaSmem) ==
                       cudaSuccess
                   ? n
                   : 0;
#define SW2D_O(id, nw, mb, un)                                                                           \
    if (variant == id &&                                                                                 \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stream_step_kernel<nw, mb, un, false, false>, nw * 32, 0) != \
            cudaSuccess)                                                                                 \
        n = 0;
    SW2D_STREAM_VARIANTS(SW2D_O)
#undef SW2D_O
    return n;
}

// Resident CTAs per SM of the build's pipelined form (every form of a build
// has the same register budget and shared memory).
int stream_pipe_ctas_per_sm(int variant) {
    if (variant == kTmaVariant) variant = 0;  // the TMA build has no pipelined form: build 0's
    int n = 0;
#define SW2D_PO(id, nw, mb, un)                                                                          \
    if (variant == id &&                                                                                 \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stream_pipe_kernel<nw, mb, un, false, false>, nw * 32, 0) != \
            cudaSuccess)                                                                                 \
        n = 0;
    SW2D_STREAM_VARIANTS(SW2D_PO)
#undef SW2D_PO
    return n;
}

int stream_pipe_max_iters() { return kPipeMaxIters; }
int stream_pipe_min_strip() { return kPipeMinStrip; }

// The plan kernel, then one cooperative launch of K iterations.
cudaError_t launch_stream_pipe(int variant, int nblocks, int tiles_w, int strip_h, int units, const GridDesc &G,
                               const ForcingDesc &F, const StateBufs<float> &S, const Thr<float> &T, Clock *clk,
                               const Control *ctl, int slot, Plan *plans, unsigned *words, unsigned *flags, int K,
                               cudaStream_t st) {
    const int strips = (G.rows + strip_h - 1) / strip_h;  // the shortest strip has rows / strips rows
    if (K < 1 || K > kPipeMaxIters || (strips > 1 && G.rows / strips < kPipeMinStrip)) return cudaErrorInvalidValue;
    pipe_plan_kernel<<<1, ((K + 31) / 32) * 32, 0, st>>>(G, F, clk, ctl, slot, plans, words, flags, units, K);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const StreamShape sh = stream_shape(G.rows, tiles_w, strip_h, units, true, 0);
    PipeDesc P;
    P.plans = plans;
    P.words = words;
    P.flags = flags;
    const bool gen = F.rain_kind == RAIN_STORM || G.n_src > 0;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // every unit resident: the waits between units end
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(nblocks);
    lc.dynamicSmemBytes = 0;
    lc.stream = st;
    lc.attrs = attr;
    lc.numAttrs = 1;
    if (variant == kTmaVariant) variant = 0;
#define SW2D_PL(id, nw, mb, un)                                                                            \
    if (variant == id) {                                                                                 \
        lc.blockDim = dim3(nw * 32);                                                                     \
        if (S.rainw && gen)                                                                              \
            return cudaLaunchKernelEx(&lc, stream_pipe_kernel<nw, mb, un, true, true>, G, F, S, T, clk, ctl, slot, sh, P);   \
        else if (S.rainw)                                                                                \
            return cudaLaunchKernelEx(&lc, stream_pipe_kernel<nw, mb, un, true, false>, G, F, S, T, clk, ctl, slot, sh, P);  \
        else if (gen)                                                                                    \
            return cudaLaunchKernelEx(&lc, stream_pipe_kernel<nw, mb, un, false, true>, G, F, S, T, clk, ctl, slot, sh, P);  \
        else                                                                                             \
            return cudaLaunchKernelEx(&lc, stream_pipe_kernel<nw, mb, un, false, false>, G, F, S, T, clk, ctl, slot, sh, P); \
    }
    SW2D_STREAM_VARIANTS(SW2D_PL)
#undef SW2D_PL
    return cudaErrorInvalidValue;
}

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry points (no link
// against the driver library)
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// Tensor map of one plane of the pitched layout, frame included, from its
// cell-(0,0) pointer: dimensions (pitch, plane rows), boxes of one row.
bool plane_map(CUtensorMap *m, const void *cell00, int rows, int pitch, bool u8) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn || !cell00) return false;
    const size_t es = u8 ? 1 : 4;
    char *base = (char *)cell00 - origin_for(pitch) * es;
    cuuint64_t dims[2] = {(cuuint64_t)pitch, (cuuint64_t)(plane_for(rows, pitch) / pitch)};
    cuuint64_t strides[1] = {(cuuint64_t)pitch * es};
    cuuint32_t box[2] = {(cuuint32_t)(u8 ? kTmaBoxM : kTmaBoxF), 1u};
    cuuint32_t estr[2] = {1u, 1u};
    return fn(m, u8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t launch_stream_step(int variant, int nblocks, int tiles_w, int strip_h, int units, int skew,
                               const GridDesc &G, const ForcingDesc &F, const StateBufs<float> &S,
                               const Thr<float> &T, Clock *clk, const Control *ctl, int slot, cudaStream_t st) {
    const StreamShape sh = stream_shape(G.rows, tiles_w, strip_h, units, false, skew);
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
    if (variant == kTmaVariant) {
        if (!S.rainw && !gen) {
            TmaMaps M;
            std::memset(&M, 0, sizeof(M));
            bool ok = true;
            for (int b = 0; b < 2; b++)
                ok = ok && plane_map(&M.h[b], S.h[b], G.rows, G.pitch, false) &&
                     plane_map(&M.um[b], S.um[b], G.rows, G.pitch, false) &&
                     plane_map(&M.vn[b], S.vn[b], G.rows, G.pitch, false) &&
                     plane_map(&M.r[b], S.hr[b], G.rows, G.pitch, false);
            ok = ok && plane_map(&M.dzx, S.dzx, G.rows, G.pitch, false) &&
                 plane_map(&M.dzy, S.dzy, G.rows, G.pitch, false) && plane_map(&M.m, S.mask, G.rows, G.pitch, true);
            if (S.nman) ok = ok && plane_map(&M.n, S.nman, G.rows, G.pitch, false);
            if (!ok) return cudaErrorInvalidValue;
            lc.blockDim = dim3(64);
            lc.dynamicSmemBytes = kTmaSmem;
            return cudaLaunchKernelEx(&lc, stream_step_tma_kernel<2, 10, 2>, G, F, S, T, clk, ctl, slot, sh, M);
        }
        variant = 0;
    }
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
