// sw2d_launch.h -- host launchers of the device kernels, one overload set per
// working precision.  The FP64 set lives in step_f64.cu (compiled without
// FMA contraction), the FP32 set in step_f32.cu (fast math).
#pragma once

#include "sw2d_device.cuh"

namespace sw2d {

// Every device field is a pitched array with a zero frame around the domain:
// kGhostTop rows above row 0, kGhostBottom rows below the south face row,
// kGhostLeft columns left of column 0 and at least 30 right of the east wall
// (the streaming kernel's last window reads 29 columns past it).
// Kernel pointers point at cell (0,0); the FP32 streaming kernel reads the
// frame instead of testing bounds (zero = inactive cell / wall, exactly the
// values the bounds tests would substitute).
constexpr int kGhostTop = 4, kGhostBottom = 4, kGhostLeft = 4;
inline int pitch_for(int cols) { return ((cols + 34 + 31) / 32) * 32; }
inline size_t plane_for(int rows, int pitch) { return (size_t)(kGhostTop + rows + 1 + kGhostBottom) * pitch; }
inline size_t origin_for(int pitch) { return (size_t)kGhostTop * pitch + kGhostLeft; }
// Kernels index a field, frame included, with 32-bit element offsets.
// (rows and cols are bounded first, so that the int sums inside pitch_for and
// plane_for cannot overflow)
inline bool plane_fits_int32(int rows, int cols) {
    return rows >= 1 && cols >= 1 && rows < (1 << 30) && cols < (1 << 30) &&
           (long long)plane_for(rows, pitch_for(cols)) < (1ll << 31);
}

// Core tiles supported by the step kernel instantiations.
bool tile_supported(int precision, int th, int tw);
void default_tile(int precision, int *th, int *tw);

#define SW2D_DECLARE_LAUNCHERS(Real)                                                                          \
    cudaError_t prepare_step(int th, int tw, Real tag);                                                      \
    cudaError_t launch_step(int th, int tw, int nblocks, const GridDesc &G, const ForcingDesc &F,             \
                            const StateBufs<Real> &S, const Thr<Real> &T, Clock *clk, const Control *ctl,    \
                            int slot, cudaStream_t st);                                                      \
    cudaError_t launch_pack_static(const double *z, const double *n, int rows, int cols, int pitch,         \
                                   double nodata, Real *zout, Real *nout, uint8_t *mask, cudaStream_t st);   \
    cudaError_t launch_pack_dz(const double *z, int rows, int cols, int pitch, const uint8_t *mask, Real *dzx, \
                               Real *dzy, cudaStream_t st);                                                  \
    cudaError_t launch_pack_depth(const double *src, int rows, int cols, int pitch, const uint8_t *mask,     \
                                  Real *dst, cudaStream_t st);                                               \
    cudaError_t launch_pack_um(const double *src, int rows, int cols, int pitch, int south_open,             \
                               const uint8_t *mask, Real *dst, cudaStream_t st);                             \
    cudaError_t launch_pack_vn(const double *src, int rows, int cols, int pitch, const uint8_t *mask,        \
                               Real *dst, cudaStream_t st);                                                  \
    cudaError_t launch_unpack(const Real *src, const Real *add, int nr, int nc, int pitch, double *dst,    \
                              cudaStream_t st);                                                          \
    cudaError_t launch_velocity(const Real *h, const Real *um, const Real *vn, int rows, int cols, int pitch, \
                                Real ge_th, double *uu, double *vv, cudaStream_t st);                        \
    cudaError_t launch_volume(const Real *h, const Real *hr, const uint8_t *mask, int rows, int cols, int pitch, \
                              double *partial, int nblocks, cudaStream_t st);                                \
    cudaError_t launch_cmax(const Real *h, const Real *um, const Real *vn, const uint8_t *mask, int rows,    \
                            int cols, int pitch, int south_open, Real ge_th, double g,                       \
                            unsigned long long *out, cudaStream_t st);                                       \
    cudaError_t launch_probe(const Real *h, const Real *hr, int rows, int cols, int pitch, const int *cells, int n, \
                             double *out, cudaStream_t st);

SW2D_DECLARE_LAUNCHERS(double)
SW2D_DECLARE_LAUNCHERS(float)

// FP32 warp-streaming step kernel (step_f32.cu)
int stream_out_cols();
int stream_variants();
int stream_warps(int variant);
int stream_ctas_per_sm(int variant);
const char *stream_variant_name(int variant);  // "stream_step_kernel<warps,minB,unroll>"  // resident CTAs per SM (occupancy), 0 on error
cudaError_t prepare_stream_step(int variant);
// skew: percent by which strip heights fall from the first strip to the last (0 = even).
cudaError_t launch_stream_step(int variant, int nblocks, int tiles_w, int strip_h, int units, int skew,
                               const GridDesc &G, const ForcingDesc &F, const StateBufs<float> &S,
                               const Thr<float> &T, Clock *clk, const Control *ctl, int slot, cudaStream_t st);

// The same kernel running several iterations per launch (fixed time step
// only; sw2d_pipe.cuh): occupancy of its pipelined form, its limits, and the
// plan kernel + cooperative launch of K iterations (plans: K entries, words:
// 2, flags: two per unit).
int stream_pipe_ctas_per_sm(int variant);
int stream_pipe_max_iters();
int stream_pipe_min_strip();
cudaError_t launch_stream_pipe(int variant, int nblocks, int tiles_w, int strip_h, int units, const GridDesc &G,
                               const ForcingDesc &F, const StateBufs<float> &S, const Thr<float> &T, Clock *clk,
                               const Control *ctl, int slot, Plan *plans, unsigned *words, unsigned *flags, int K,
                               cudaStream_t st);

constexpr int kVolumeBlocks = 1024;
constexpr int kVolumeThreads = 256;

}  // namespace sw2d
