// sw2d_launch_impl.cuh -- bodies of the launchers declared in sw2d_launch.h,
// included once per precision translation unit with SW2D_REAL defined.
#pragma once

#include "sw2d_aux.cuh"
#include "sw2d_device.cuh"
#include "sw2d_launch.h"

namespace sw2d {
namespace detail {

inline int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int)b;
}

// Raises the dynamic shared-memory limit of one instantiation; called when a
// handle is created (on its device), never inside a stream capture.
template <class Real, int TH, int TW, int NT>
cudaError_t step_prepare() {
    constexpr size_t smem = step_smem_bytes<Real, TH, TW>();
    cudaError_t e = cudaFuncSetAttribute(step_kernel<Real, TH, TW, NT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // all of the unified L1/shared storage as shared memory: more resident CTAs
    return cudaFuncSetAttribute(step_kernel<Real, TH, TW, NT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared);
}

template <class Real, int TH, int TW, int NT>
cudaError_t step_launch(int nblocks, const GridDesc &G, const ForcingDesc &F, const StateBufs<Real> &S,
                        const Thr<Real> &T, Clock *clk, const Control *ctl, int slot, cudaStream_t st) {
    constexpr size_t smem = step_smem_bytes<Real, TH, TW>();
    step_kernel<Real, TH, TW, NT><<<nblocks, NT, smem, st>>>(G, F, S, T, clk, ctl, slot);
    return cudaGetLastError();
}

}  // namespace detail

cudaError_t launch_pack_static(const double *z, const double *n, int rows, int cols, int pitch, double nodata,
                               SW2D_REAL *zout, SW2D_REAL *nout, uint8_t *mask, cudaStream_t st) {
    pack_static_kernel<SW2D_REAL><<<detail::grid_for((long long)rows * cols, 256), 256, 0, st>>>(
        z, n, rows, cols, pitch, nodata, zout, nout, mask);
    return cudaGetLastError();
}

cudaError_t launch_pack_dz(const double *z, int rows, int cols, int pitch, const uint8_t *mask, SW2D_REAL *dzx,
                           SW2D_REAL *dzy, cudaStream_t st) {
    pack_dz_kernel<SW2D_REAL><<<detail::grid_for((long long)rows * cols, 256), 256, 0, st>>>(z, rows, cols, pitch, mask,
                                                                                           dzx, dzy);
    return cudaGetLastError();
}

cudaError_t launch_pack_depth(const double *src, int rows, int cols, int pitch, const uint8_t *mask,
                              SW2D_REAL *dst, cudaStream_t st) {
    pack_depth_kernel<SW2D_REAL><<<detail::grid_for((long long)rows * cols, 256), 256, 0, st>>>(
        src, rows, cols, pitch, mask, dst);
    return cudaGetLastError();
}

cudaError_t launch_pack_um(const double *src, int rows, int cols, int pitch, int south_open,
                           const uint8_t *mask, SW2D_REAL *dst, cudaStream_t st) {
    pack_um_kernel<SW2D_REAL><<<detail::grid_for((long long)(rows + 1) * cols, 256), 256, 0, st>>>(
        src, rows, cols, pitch, south_open, mask, dst);
    return cudaGetLastError();
}

cudaError_t launch_pack_vn(const double *src, int rows, int cols, int pitch, const uint8_t *mask,
                           SW2D_REAL *dst, cudaStream_t st) {
    pack_vn_kernel<SW2D_REAL><<<detail::grid_for((long long)rows * (cols + 1), 256), 256, 0, st>>>(
        src, rows, cols, pitch, mask, dst);
    return cudaGetLastError();
}

cudaError_t launch_unpack(const SW2D_REAL *src, const SW2D_REAL *add, int nr, int nc, int pitch, double *dst,
                          cudaStream_t st) {
    unpack_kernel<SW2D_REAL><<<detail::grid_for((long long)nr * nc, 256), 256, 0, st>>>(src, add, nr, nc, pitch, dst);
    return cudaGetLastError();
}

cudaError_t launch_velocity(const SW2D_REAL *h, const SW2D_REAL *um, const SW2D_REAL *vn, int rows, int cols,
                            int pitch, SW2D_REAL ge_th, double *uu, double *vv, cudaStream_t st) {
    velocity_kernel<SW2D_REAL><<<detail::grid_for((long long)rows * cols, 256), 256, 0, st>>>(
        h, um, vn, rows, cols, pitch, ge_th, uu, vv);
    return cudaGetLastError();
}

cudaError_t launch_volume(const SW2D_REAL *h, const SW2D_REAL *hr, const uint8_t *mask, int rows, int cols, int pitch,
                          double *partial, int nblocks, cudaStream_t st) {
    volume_kernel<SW2D_REAL, kVolumeThreads><<<nblocks, kVolumeThreads, 0, st>>>(h, hr, mask, rows, cols, pitch,
                                                                                  partial);
    return cudaGetLastError();
}

cudaError_t launch_cmax(const SW2D_REAL *h, const SW2D_REAL *um, const SW2D_REAL *vn, const uint8_t *mask,
                        int rows, int cols, int pitch, int south_open, SW2D_REAL ge_th, double g,
                        unsigned long long *out, cudaStream_t st) {
    cmax_kernel<SW2D_REAL><<<detail::grid_for((long long)rows * cols, 256), 256, 0, st>>>(
        h, um, vn, mask, rows, cols, pitch, south_open, ge_th, g, out);
    return cudaGetLastError();
}

cudaError_t launch_probe(const SW2D_REAL *h, const SW2D_REAL *hr, int rows, int cols, int pitch, const int *cells,
                         int n, double *out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    probe_kernel<SW2D_REAL><<<(n + 255) / 256, 256, 0, st>>>(h, hr, rows, cols, pitch, cells, n, out);
    return cudaGetLastError();
}

}  // namespace sw2d
