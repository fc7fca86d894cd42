// sw2d_aux.cuh -- small kernels around the step kernel: converting host
// rasters (compact float64, north row first) into the pitched device layout
// of the working precision, and deriving output fields on demand.
//
// Device layout: every field is a (rows+1) x pitch array, pitch a multiple of
// 32 elements and >= cols+1.  Cell (i,j), the x-face north of it and the
// y-face west of it share the offset i*pitch+j.  Row `rows` holds the south
// boundary faces, column `cols` the east wall faces; everything else beyond
// the domain stays zero.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sw2d {

// z, optional Manning raster and the active mask (init_inf, cu:29-49:
// a cell is active when its elevation differs from NODATA, compared in FP64)
template <class Real>
__global__ void pack_static_kernel(const double *__restrict__ z, const double *__restrict__ n, int rows,
                                   int cols, int pitch, double nodata, Real *__restrict__ zout,
                                   Real *__restrict__ nout, uint8_t *__restrict__ mask) {
    const long long total = (long long)rows * cols;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / cols), j = (int)(k - (k / cols) * cols);
        const size_t gp = (size_t)i * pitch + j;
        const double zv = z[k];
        mask[gp] = (zv != nodata) ? 1 : 0;
        zout[gp] = (Real)zv;
        if (nout) nout[gp] = (Real)(n ? n[k] : 0.0);
    }
}

// depth; inactive cells hold 0 (the reference zeroes them in its first
// continuity call, cu:658-660, and reads them nowhere before that)
template <class Real>
__global__ void pack_depth_kernel(const double *__restrict__ src, int rows, int cols, int pitch,
                                  const uint8_t *__restrict__ mask, Real *__restrict__ dst) {
    const long long total = (long long)rows * cols;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / cols), j = (int)(k - (k / cols) * cols);
        const size_t gp = (size_t)i * pitch + j;
        const Real v = mask[gp] ? (Real)src[k] : Real(0);
        dst[gp] = v;
        // the frame row below the last cell row holds a copy of its depth (the
        // streaming kernel's face depth at the south face); the tile kernel
        // and every other reader stop at row rows-1
        if (i == rows - 1) dst[gp + pitch] = v;
    }
}

// Bed-elevation differences across the faces, for the FP32 streaming kernel:
// dzx(i,j) = z(i,j) - z(i-1,j) on the x-face north of cell (i,j) and
// dzy(i,j) = z(i,j) - z(i,j-1) on the y-face west of it, formed in FP64 from
// the float64 DEM and rounded once; 0 on faces that are not between two active
// cells.  The scheme uses the bed only through such differences (surface
// slopes and the dry-bed rules), and a difference of a few centimetres taken
// between two FP32 elevations near 100 m would carry their rounding (about
// 4 um each) into every slope.
template <class Real>
__global__ void pack_dz_kernel(const double *__restrict__ z, int rows, int cols, int pitch,
                               const uint8_t *__restrict__ mask, Real *__restrict__ dzx, Real *__restrict__ dzy) {
    const long long total = (long long)rows * cols;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / cols), j = (int)(k - (k / cols) * cols);
        const size_t gp = (size_t)i * pitch + j;
        const bool m = mask[gp] != 0;
        dzx[gp] = (i > 0 && m && mask[gp - pitch]) ? (Real)(z[k] - z[k - cols]) : Real(0);
        dzy[gp] = (j > 0 && m && mask[gp - 1]) ? (Real)(z[k] - z[k - 1]) : Real(0);
    }
}

// x-faces (rows+1) x cols.  A face is open only between two active cells or,
// with an open south edge, below an active last-row cell; others are walls.
template <class Real>
__global__ void pack_um_kernel(const double *__restrict__ src, int rows, int cols, int pitch, int south_open,
                               const uint8_t *__restrict__ mask, Real *__restrict__ dst) {
    const long long total = (long long)(rows + 1) * cols;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / cols), j = (int)(k - (k / cols) * cols);
        const size_t gp = (size_t)i * pitch + j;
        bool open;
        if (i == 0) open = false;
        else if (i == rows) open = south_open && mask[gp - pitch];
        else open = mask[gp] && mask[gp - pitch];
        dst[gp] = (open && src) ? (Real)src[k] : Real(0);
    }
}

// y-faces rows x (cols+1); the west and east edges are walls
template <class Real>
__global__ void pack_vn_kernel(const double *__restrict__ src, int rows, int cols, int pitch,
                               const uint8_t *__restrict__ mask, Real *__restrict__ dst) {
    const long long total = (long long)rows * (cols + 1);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / (cols + 1)), j = (int)(k - (k / (cols + 1)) * (cols + 1));
        const size_t gp = (size_t)i * pitch + j;
        const bool open = j > 0 && j < cols && mask[gp] && mask[gp - 1];
        dst[gp] = (open && src) ? (Real)src[k] : Real(0);
    }
}

// nr x nc window of a pitched array -> compact float64
template <class Real>
__global__ void unpack_kernel(const Real *__restrict__ src, const Real *__restrict__ add, int nr, int nc, int pitch,
                              double *__restrict__ dst) {
    const long long total = (long long)nr * nc;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / nc), j = (int)(k - (k / nc) * nc);
        const size_t gp = (size_t)i * pitch + j;
        dst[k] = (double)src[gp] + (add ? (double)add[gp] : 0.0);  // add: the depth's remainder plane
    }
}

// face velocity with the reference's face-depth rules (cu:374-394, cu:418-430)
template <class Real>
__device__ __forceinline__ Real face_vel_x(const Real *h, const Real *um, int i, int j, int rows, int pitch,
                                           Real ge_th) {
    const size_t gp = (size_t)i * pitch + j;
    Real hm;
    if (i == 0) hm = h[gp];
    else if (i == rows) hm = h[gp - pitch];
    else hm = Real(0.50) * (h[gp] + h[gp - pitch]);
    return (hm >= ge_th) ? um[gp] / hm : Real(0.00);
}

template <class Real>
__device__ __forceinline__ Real face_vel_y(const Real *h, const Real *vn, int i, int j, int cols, int pitch,
                                           Real ge_th) {
    const size_t gp = (size_t)i * pitch + j;
    Real hn;
    if (j == 0) hn = h[gp];
    else if (j == cols) hn = h[gp - 1];
    else hn = Real(0.50) * (h[gp] + h[gp - 1]);
    return (hn >= ge_th) ? vn[gp] / hn : Real(0.0);
}

// cell velocities (uu_vv, cu:459-484): uu along rows, vv along columns
template <class Real>
__global__ void velocity_kernel(const Real *__restrict__ h, const Real *__restrict__ um, const Real *__restrict__ vn,
                                int rows, int cols, int pitch, Real ge_th, double *__restrict__ uu,
                                double *__restrict__ vv) {
    const long long total = (long long)rows * cols;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / cols), j = (int)(k - (k / cols) * cols);
        const size_t gp = (size_t)i * pitch + j;
        if (h[gp] >= ge_th) {
            const Real a = (face_vel_x(h, um, i + 1, j, rows, pitch, ge_th) + face_vel_x(h, um, i, j, rows, pitch, ge_th)) / Real(2.00);
            const Real b = (face_vel_y(h, vn, i, j + 1, cols, pitch, ge_th) + face_vel_y(h, vn, i, j, cols, pitch, ge_th)) / Real(2.00);
            uu[k] = (double)a;
            vv[k] = (double)b;
        } else {
            uu[k] = 0.0;
            vv[k] = 0.0;
        }
    }
}

// per-block FP64 partial sums of the depth on active cells.  Fixed grid and
// fixed per-thread order, so the result is deterministic; the host adds the
// partials with Kahan summation.
template <class Real, int NT>
__global__ void __launch_bounds__(NT) volume_kernel(const Real *__restrict__ h, const Real *__restrict__ hr,
                                                    const uint8_t *__restrict__ mask,
                                                    int rows, int cols, int pitch, double *__restrict__ partial) {
    __shared__ double s[NT / 32];
    const long long total = (long long)rows * cols;
    double acc = 0.0, comp = 0.0;
    for (long long k = blockIdx.x * (long long)NT + threadIdx.x; k < total; k += (long long)gridDim.x * NT) {
        const int i = (int)(k / cols), j = (int)(k - (k / cols) * cols);
        const size_t gp = (size_t)i * pitch + j;
        if (mask[gp]) {
            const double y = ((double)h[gp] + (hr ? (double)hr[gp] : 0.0)) - comp;
            const double t = acc + y;
            comp = (t - acc) - y;
            acc = t;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < NT / 32; w++) v += s[w];
        partial[blockIdx.x] = v;
    }
}

// CFL speed bound of a state (the rule of the step kernel's stage 5)
template <class Real>
__global__ void cmax_kernel(const Real *__restrict__ h, const Real *__restrict__ um, const Real *__restrict__ vn,
                            const uint8_t *__restrict__ mask, int rows, int cols, int pitch, int south_open,
                            Real ge_th, double g, unsigned long long *__restrict__ out) {
    const long long total = (long long)rows * cols;
    Real cm = 0;
    const Real gr = (Real)g;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / cols), j = (int)(k - (k / cols) * cols);
        const size_t gp = (size_t)i * pitch + j;
        if (!mask[gp]) continue;
        if (i > 0 && mask[gp - pitch]) {
            const Real hm = Real(0.50) * (h[gp] + h[gp - pitch]);
            if (hm >= ge_th) cm = fmax(cm, fabs(um[gp] / hm) + sqrt(gr * hm));
        }
        if (i == rows - 1 && south_open) {
            const Real hm = h[gp];
            if (hm >= ge_th) cm = fmax(cm, fabs(um[gp + pitch] / hm) + sqrt(gr * hm));
        }
        if (j > 0 && mask[gp - 1]) {
            const Real hn = Real(0.50) * (h[gp] + h[gp - 1]);
            if (hn >= ge_th) cm = fmax(cm, fabs(vn[gp] / hn) + sqrt(gr * hn));
        }
    }
    double v = (double)cm;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(v));
}

template <class Real>
__global__ void probe_kernel(const Real *__restrict__ h, const Real *__restrict__ hr, int rows, int cols, int pitch,
                             const int *__restrict__ cells, int n, double *__restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int c = cells[k];
    if (c < 0 || c >= rows * cols) {
        out[k] = 0.0;
        return;
    }
    const int i = c / cols, j = c - (c / cols) * cols;
    const size_t gp = (size_t)i * pitch + j;
    out[k] = (double)h[gp] + (hr ? (double)hr[gp] : 0.0);
}

}  // namespace sw2d
