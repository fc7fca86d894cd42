// sw2d_noalloc.cu -- the mass-balance volume sum for callers that must not
// allocate device memory.
//
// sw2d_get_budget sums the depth field with volume_kernel into a partial-sum
// buffer the handle allocated with cudaMalloc.  Some callers cannot allocate
// at the point where they need that check: a host model whose own memory
// pool has already reserved the whole device (a cudaMalloc there fails, or
// makes the pool give memory back), or one that must not call the allocator
// inside its time loop (cudaMalloc and cudaFree can synchronise the device).
// sw2d_volume_noalloc runs the same kind of reduction on device arrays the
// caller passes in, keeping its partial sums in a fixed array that is part of
// this library's device image instead.
//
// Scratch: g_volume_scratch, kNoallocMaxChunks + 1 doubles (64 KiB), resident
// on every GPU that loads the library until the process exits.  Chunk b holds
// the sum of cells [b*kNoallocChunk, (b+1)*kNoallocChunk) in row-major order;
// the last element receives the total.  Every call overwrites the partials it
// uses, so nothing has to start at zero; calls that overlap on the GPU
// (different streams, or different host threads) share the array and race.
//
// Set-up: host code cannot use the array's name as a device address, so the
// first call in a CUDA context (per device, and again after the context was
// destroyed and made anew, e.g. by cudaDeviceReset) looks the address up with
// cudaGetSymbolAddress, with that device current, and keeps it for the
// context's lifetime.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sw2d.h"

namespace {

constexpr int kNoallocChunk = 8192;                                   // cells per CTA
constexpr int kNoallocMaxChunks = SW2D_NOALLOC_MAX_CELLS / kNoallocChunk;  // 8192
constexpr int kNoallocThreads = 256;
constexpr int kMaxDevices = 64;

static_assert((long long)kNoallocMaxChunks * kNoallocChunk == SW2D_NOALLOC_MAX_CELLS, "chunking");

static __device__ __align__(256) double g_volume_scratch[kNoallocMaxChunks + 1];

// Deterministic: fixed cells per CTA, fixed order per thread (Kahan), fixed
// shuffle tree and warp order.
__global__ void __launch_bounds__(kNoallocThreads)
    noalloc_volume_chunks(const double *__restrict__ h, const uint8_t *__restrict__ mask, int rows, int cols,
                          int pitch, long long ncells, double *__restrict__ partial) {
    __shared__ double s[kNoallocThreads / 32];
    const long long first = (long long)blockIdx.x * kNoallocChunk;
    long long last = first + kNoallocChunk;
    if (last > ncells) last = ncells;
    double acc = 0.0, comp = 0.0;
    for (long long k = first + threadIdx.x; k < last; k += kNoallocThreads) {
        const int i = (int)(k / cols), j = (int)(k - (k / cols) * cols);
        const size_t gp = (size_t)i * pitch + j;
        if (mask == nullptr || mask[gp]) {
            const double y = h[gp] - comp;
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
        for (int w = 0; w < kNoallocThreads / 32; w++) v += s[w];
        partial[blockIdx.x] = v;
    }
    (void)rows;
}

// One thread adds the chunk sums in chunk order (Kahan) into partial[n].
__global__ void noalloc_volume_total(double *__restrict__ partial, int n) {
    double s = 0.0, c = 0.0;
    for (int b = 0; b < n; b++) {
        const double y = partial[b] - c;
        const double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    partial[kNoallocMaxChunks] = s;
}

std::mutex g_setup_mutex;

// The scratch address of each device, with the context it is valid in.
struct ScratchEntry {
    unsigned long long ctx_id;  // cuCtxGetId of the context (never reused in a process); 0 = none
    double *ptr;
};
ScratchEntry g_scratch[kMaxDevices] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// The identity of the current context through the driver's entry points (no
// link against the driver library); 0 when there is none or it cannot be
// told.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
        looked_up = true;
    }
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array in the current context: looked up once
// per context (cudaGetSymbolAddress with the device current) and kept.
cudaError_t scratch_for_current_device(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    const unsigned long long id = current_context_id();
    if (id != 0 && g_scratch[dev].ctx_id == id && g_scratch[dev].ptr != nullptr) {
        *out = g_scratch[dev].ptr;
        return cudaSuccess;
    }
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_volume_scratch);  // also makes the device's primary context current
    if (e != cudaSuccess) return e;
    // keyed on the context now current; when it cannot be told, nothing is
    // kept and the next call looks the address up again
    g_scratch[dev].ctx_id = current_context_id();
    g_scratch[dev].ptr = g_scratch[dev].ctx_id != 0 ? static_cast<double *>(p) : nullptr;
    *out = static_cast<double *>(p);
    return cudaSuccess;
}

}  // namespace

extern "C" int sw2d_volume_noalloc(const double *depth, const uint8_t *mask, int32_t rows, int32_t cols,
                                   int32_t pitch, double cell_area, void *stream, double *volume_out) {
    if (!depth || !volume_out || rows < 1 || cols < 1 || pitch < cols || !(cell_area > 0.0))
        return SW2D_ERR_INVALID_ARG;
    const long long ncells = (long long)rows * cols;
    if (ncells > SW2D_NOALLOC_MAX_CELLS) return SW2D_ERR_INVALID_ARG;  // beyond the scratch array
    double *scratch = nullptr;
    if (scratch_for_current_device(&scratch) != cudaSuccess) return SW2D_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    (void)cudaGetLastError();  // an earlier, unrelated launch error is not this call's
    const int nchunks = (int)((ncells + kNoallocChunk - 1) / kNoallocChunk);
    noalloc_volume_chunks<<<nchunks, kNoallocThreads, 0, st>>>(depth, mask, rows, cols, pitch, ncells, scratch);
    if (cudaGetLastError() != cudaSuccess) return SW2D_ERR_CUDA;
    noalloc_volume_total<<<1, 1, 0, st>>>(scratch, nchunks);
    if (cudaGetLastError() != cudaSuccess) return SW2D_ERR_CUDA;
    double sum = 0.0;
    if (cudaMemcpyAsync(&sum, scratch + kNoallocMaxChunks, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return SW2D_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return SW2D_ERR_CUDA;
    *volume_out = sum * cell_area;
    return SW2D_OK;
}
