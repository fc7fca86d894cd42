// sw2d_api.cu -- host implementation of the C ABI declared in include/sw2d.h.
//
// A handle owns: the pitched device state in two ping-pong buffers (h, um,
// vn), the static fields, a float64 staging buffer for uploads/downloads,
// three rotating Clock slots, the Control block, the forcing tables, one
// non-blocking stream and a CUDA graph of kChunk step launches that is
// replayed by sw2d_advance.  Time and time step live on the device, so an
// advance needs one host synchronisation per chunk, not per iteration (the
// reference synchronises nine times per iteration, cu:1268-1332).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sw2d.h"
#include "sw2d_launch.h"

using namespace sw2d;

namespace {

constexpr int kChunk = 48;  // launches per graph replay, a multiple of 3 (clock slots)

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct sw2d_handle {
    sw2d_config cfg{};
    int real_size = 8;
    int pitch = 0;
    size_t plane = 0;   // elements per allocated array, frame included
    size_t origin = 0;  // element offset of cell (0,0) in an allocation
    int tile_h = 16, tile_w = 32, nblocks = 0;
    bool stream_kernel = false;  // FP32 warp-streaming kernel instead of the tile kernel
    int strip_h = 0, stream_tiles_w = 0, stream_units = 0, variant = 0;
    int strip_skew = 0;  // percent by which strip heights fall from the first strip to the last
    cudaStream_t stream = nullptr;
    void *h[2] = {nullptr, nullptr}, *um[2] = {nullptr, nullptr}, *vn[2] = {nullptr, nullptr};
    void *z = nullptr, *nman = nullptr;
    uint8_t *mask = nullptr;
    void *rainw = nullptr;  // spatial rain factors (allocated on first use)
    void *dzx = nullptr, *dzy = nullptr;  // bed differences across faces (streaming kernel)
    void *hr[2] = {nullptr, nullptr};      // depth remainders of the compensated FP32 state (streaming kernel)
    bool use_rainw = false;
    double *stage = nullptr, *stage2 = nullptr;
    size_t stage_elems = 0;
    double *partial = nullptr;
    Clock *d_clk = nullptr;
    Control *d_ctl = nullptr;
    Clock *h_clk = nullptr;    // pinned
    Control *h_ctl = nullptr;  // pinned
    double *h_partial = nullptr;  // pinned
    DevBuf rain, ev, src_cell, src_q, probe_cells, probe_out;
    ForcingDesc F{};
    GridDesc G{};
    bool have_static = false, have_state = false, has_nraster = false;
    long long launches = 0;  // clock-slot rotations (one per launch that finalises a slot)
    long long kernels = 0;   // kernel launches of the time loop
    // several iterations per launch (fixed time step, streaming kernel):
    // iterations per launch (0 = one launch per iteration), the plan table,
    // its run count and abort word, and the per-unit progress counters
    int pipe_k = 0;
    bool pipe_auto = false;    // pipe_k is the library's choice (steps_per_launch = 0)
    bool fold_needed = false;  // one-iteration launches left a budget fold to do (read_clock)
    Plan *d_plans = nullptr;
    unsigned *d_words = nullptr;
    unsigned *d_flags = nullptr;
    Clock clock{};  // last clock read back
    double volume0 = 0.0;
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    std::string err;
};

namespace {

int fail(sw2d_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    return code;
}

int cuda_fail(sw2d_handle *h, cudaError_t e, const char *what) {
    const int code = (e == cudaErrorMemoryAllocation) ? SW2D_ERR_OOM : SW2D_ERR_CUDA;
    return fail(h, code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(h, expr)                                             \
    do {                                                        \
        cudaError_t e_ = (expr);                                \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #expr); \
    } while (0)

bool is_f64(const sw2d_handle *h) { return h->cfg.precision == SW2D_PREC_F64; }

// start of the allocation of a state field (its frame included)
void *raw_field(const sw2d_handle *h, void *p) { return static_cast<char *>(p) - h->origin * h->real_size; }

template <class Real>
Real thr_ge(double x) {
    if (sizeof(Real) == 8) return (Real)x;
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, INFINITY);
    return (Real)f;
}

template <class Real>
Real thr_gt(double x) {
    if (sizeof(Real) == 8) return (Real)std::nextafter(x, INFINITY);
    float f = (float)x;
    if ((double)f <= x) f = std::nextafter(f, INFINITY);
    return (Real)f;
}

template <class Real>
Thr<Real> make_thr(const sw2d_config &c) {
    Thr<Real> t;
    t.gt_th = thr_gt<Real>(c.th);
    t.ge_th = thr_ge<Real>(c.th);
    t.gt_evmin = thr_gt<Real>(c.EV_WL_min);
    return t;
}

template <class Real>
StateBufs<Real> make_bufs(const sw2d_handle *h) {
    StateBufs<Real> s;
    for (int b = 0; b < 2; b++) {
        s.h[b] = (Real *)h->h[b];
        s.um[b] = (Real *)h->um[b];
        s.vn[b] = (Real *)h->vn[b];
    }
    s.z = (const Real *)h->z;
    s.nman = h->has_nraster ? (const Real *)h->nman : nullptr;
    s.mask = h->mask;
    s.rainw = h->use_rainw ? (const Real *)h->rainw : nullptr;
    s.hr[0] = (Real *)h->hr[0];
    s.hr[1] = (Real *)h->hr[1];
    s.dzx = (const Real *)h->dzx;
    s.dzy = (const Real *)h->dzy;
    return s;
}

cudaError_t launch_one(sw2d_handle *h, int slot) {
    if (h->stream_kernel)
        return launch_stream_step(h->variant, h->nblocks, h->stream_tiles_w, h->strip_h, h->stream_units,
                                  h->strip_skew, h->G, h->F,
                                  make_bufs<float>(h), make_thr<float>(h->cfg), h->d_clk, h->d_ctl, slot, h->stream);
    if (is_f64(h))
        return launch_step(h->tile_h, h->tile_w, h->nblocks, h->G, h->F, make_bufs<double>(h),
                           make_thr<double>(h->cfg), h->d_clk, h->d_ctl, slot, h->stream);
    return launch_step(h->tile_h, h->tile_w, h->nblocks, h->G, h->F, make_bufs<float>(h),
                       make_thr<float>(h->cfg), h->d_clk, h->d_ctl, slot, h->stream);
}

// Whether advance runs several iterations per launch now: the pipelined form
// with the storm or point sources compiled in spills at 96 registers and
// measured 0.86-0.94x one launch per iteration on 256^2 to 1024^2, so the
// library's own choice of it (not one the caller asked for) stands down
// while that forcing is set.
bool pipe_now(const sw2d_handle *h) {
    if (h->pipe_k <= 0) return false;
    const bool gen = h->F.rain_kind == RAIN_STORM || h->G.n_src > 0;
    return !(h->pipe_auto && gen);
}

int validate(const sw2d_config *c, std::string *why) {
    if (!c) return *why = "config is null", 0;
    if (c->rows < 1 || c->cols < 1) return *why = "rows and cols must be >= 1", 0;
    if (!plane_fits_int32(c->rows, c->cols)) return *why = "grid too large for 32-bit indexing", 0;
    if (!(c->dx > 0) || !(c->dy > 0)) return *why = "dx and dy must be > 0", 0;
    if (!(c->dt > 0)) return *why = "dt must be > 0", 0;
    if (c->precision != SW2D_PREC_F64 && c->precision != SW2D_PREC_F32) return *why = "unknown precision", 0;
    if (c->dt_mode != SW2D_DT_FIXED && c->dt_mode != SW2D_DT_CFL) return *why = "unknown dt_mode", 0;
    if (c->dt_mode == SW2D_DT_CFL && !(c->cfl > 0)) return *why = "cfl must be > 0", 0;
    if (!(c->g > 0) || !(c->th >= 0)) return *why = "g must be > 0 and th >= 0", 0;
    if (c->kernel < SW2D_KERNEL_AUTO || c->kernel > SW2D_KERNEL_STREAM) return *why = "unknown kernel", 0;
    if (c->kernel == SW2D_KERNEL_STREAM && c->precision != SW2D_PREC_F32)
        return *why = "the streaming kernel is FP32 only", 0;
    if (c->strip_h < 0) return *why = "strip_h must be >= 0", 0;
    if (c->variant < 0 || c->variant >= stream_variants()) return *why = "unknown kernel variant", 0;
    if (c->steps_per_launch < 0 || c->steps_per_launch > stream_pipe_max_iters())
        return *why = "steps_per_launch must be in 0..1024", 0;
    if (c->steps_per_launch > 1 &&
        (c->dt_mode != SW2D_DT_FIXED || c->precision != SW2D_PREC_F32 || c->kernel == SW2D_KERNEL_TILE))
        return *why = "steps_per_launch > 1 needs the FP32 streaming kernel and SW2D_DT_FIXED", 0;
    return 1;
}

void grid_shape(const sw2d_config *c, int *pitch, size_t *plane, int *th, int *tw) {
    *pitch = pitch_for(c->cols);
    *plane = plane_for(c->rows, *pitch);
    int a = c->tile_h, b = c->tile_w;
    if (a <= 0 || b <= 0 || !tile_supported(c->precision, a, b)) default_tile(c->precision, &a, &b);
    *th = a;
    *tw = b;
}

int read_clock(sw2d_handle *h) {
    const int slot = (int)(h->launches % 3);
    // the streaming kernel leaves the budget fold of the slot its last
    // launch wrote to the next launch (finish_cta_deferred_warp): fold it
    // here (a fold is idempotent)
    if (h->stream_kernel && h->fold_needed && h->have_state) {
        fold_kernel<<<1, 32, 0, h->stream>>>(h->d_clk, slot, (slot + 2) % 3);
        CK(h, cudaGetLastError());
        h->kernels++;
        h->fold_needed = false;
    }
    CK(h, cudaMemcpyAsync(h->h_clk, h->d_clk + slot, sizeof(Clock), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->clock = *h->h_clk;
    return SW2D_OK;
}

int capture_graph(sw2d_handle *h) {
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int m = 0; m < kChunk && e == cudaSuccess; m++) e = launch_one(h, m % 3);
    cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(h, e, "step launch during capture");
    }
    if (e2 != cudaSuccess) return cuda_fail(h, e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
    h->graph_valid = true;
    return SW2D_OK;
}

void sync_grid_scalars(GridDesc &G) {
    G.sd.rdx = 1.0 / G.sd.dx;
    G.sd.rdy = 1.0 / G.sd.dy;
    G.sf.rdx = (float)G.sd.rdx;
    G.sf.rdy = (float)G.sd.rdy;
    G.sf.dx = (float)G.sd.dx;
    G.sf.dy = (float)G.sd.dy;
    G.sf.g = (float)G.sd.g;
    G.sf.manning = (float)G.sd.manning;
    G.sf.pct_hi = (float)G.sd.pct_hi;
    G.sf.pct_lo = (float)G.sd.pct_lo;
    G.sf.storm_amp = (float)G.sd.storm_amp;
    G.sf.storm_2s2 = (float)G.sd.storm_2s2;
}

template <class T>
int upload_table(sw2d_handle *h, DevBuf &b, const T *src, size_t n) {
    const size_t bytes = n * sizeof(T);
    if (bytes > b.bytes) {
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
        CK(h, cudaMalloc(&b.p, bytes));
        b.bytes = bytes;
    }
    if (bytes) CK(h, cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return SW2D_OK;
}

// Strip height of the FP32 streaming kernel when the caller leaves it to the
// library.  Units (column tile x strip) are sized so that a whole number of
// waves of resident warps covers the grid -- a partial last wave leaves SMs
// idle -- using the fewest waves whose strips are at most kMaxAutoStrip rows
// (longer strips measured slower on GB300 at 4096^2 and up), and at least 16
// rows, since each strip recomputes 7 halo rows.
constexpr long long kMaxAutoStrip = 160;

// Longest one-wave strip for which the library picks several iterations per
// launch by itself (steps_per_launch = 0).
constexpr int kAutoPipeMaxStrip = 32;

// Skew of the strip heights for one launch per iteration over a full wave
// (strip_rows in sw2d_stream.cuh): measured 0 / 10 / 20 / 35 % at 2048^2:
// 80.7 / 80.6 / 79.4 / 84.0 us per iteration.
constexpr int kStripSkew = 20;

int auto_strip(int rows, int tiles_w, int variant, int device) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int per_sm = stream_ctas_per_sm(variant);
    const long long resident = (long long)(sms > 0 ? sms : 152) * (per_sm > 0 ? per_sm : 1) * stream_warps(variant);
    const long long tw = tiles_w > 0 ? tiles_w : 1;
    if (resident < tw) return 64;
    long long sh = rows;
    for (long long w = 1; w == 1 || sh > kMaxAutoStrip; w++) {
        const long long k = w * resident / tw;  // strips per column tile that fill w waves
        sh = (rows + k - 1) / k;
    }
    return (int)(sh < 16 ? 16 : sh);
}

// Strip height of the pipelined launches: every unit must be resident at
// once (one wave), so strips are the shortest that fit one wave, at least 16
// rows.  0 when even one-row strips would not fit.
int pipe_strip(int rows, int tiles_w, long long resident) {
    const long long tw = tiles_w > 0 ? tiles_w : 1;
    const long long per_tile = resident / tw;  // strips per column tile that one wave holds
    if (per_tile < 1) return 0;
    const long long sh = (rows + per_tile - 1) / per_tile;
    return (int)(sh < 16 ? 16 : sh);
}

}  // namespace

namespace sw2d {

bool tile_supported(int precision, int th, int tw) {
    if (precision == SW2D_PREC_F64) return (th == 16 && tw == 32) || (th == 8 && tw == 32);
    return (th == 16 && tw == 32) || (th == 32 && tw == 32) || (th == 16 && tw == 64);
}

void default_tile(int precision, int *th, int *tw) {
    *th = precision == SW2D_PREC_F64 ? 16 : 32;
    *tw = 32;
}

}  // namespace sw2d

extern "C" {

int sw2d_config_init(sw2d_config *c) {
    if (!c) return SW2D_ERR_INVALID_ARG;
    std::memset(c, 0, sizeof(*c));
    c->rows = c->cols = 0;
    c->dx = c->dy = 1.0;
    c->nodata = -9999.0;
    c->g = 9.80;      // cu:809
    c->th = 1.0e-4;   // cu:1130
    c->manning = 0.0;
    c->precision = SW2D_PREC_F64;
    c->dt_mode = SW2D_DT_FIXED;
    c->dt = 0.04;
    c->cfl = 0.5;
    return SW2D_OK;
}

int sw2d_device_bytes(const sw2d_config *c, int64_t *bytes) {
    std::string why;
    if (!bytes || !validate(c, &why)) return SW2D_ERR_INVALID_ARG;
    int pitch, th, tw;
    size_t plane;
    grid_shape(c, &pitch, &plane, &th, &tw);
    const size_t rs = c->precision == SW2D_PREC_F64 ? 8 : 4;
    const bool stream = c->precision == SW2D_PREC_F32 && c->kernel != SW2D_KERNEL_TILE;
    size_t total = plane * rs * (stream ? 12 : 8);  // 2x(h, um, vn) + z + n (+ dzx, dzy, 2x remainder), frame included
    total += plane;                 // mask
    total += 2 * (size_t)(c->rows + 1) * (c->cols + 1) * sizeof(double);  // staging
    total += kVolumeBlocks * sizeof(double) + 3 * sizeof(Clock) + sizeof(Control);
    *bytes = (int64_t)total;
    return SW2D_OK;
}

int sw2d_create(const sw2d_config *cfg, sw2d_handle **out) {
    if (!out) return SW2D_ERR_INVALID_ARG;
    *out = nullptr;
    std::string why;
    if (!validate(cfg, &why)) return SW2D_ERR_INVALID_ARG;
    sw2d_handle *h = new (std::nothrow) sw2d_handle();  // no exception crosses the C ABI
    if (!h) return SW2D_ERR_OOM;
    h->cfg = *cfg;
    h->real_size = cfg->precision == SW2D_PREC_F64 ? 8 : 4;
    grid_shape(cfg, &h->pitch, &h->plane, &h->tile_h, &h->tile_w);
    h->origin = origin_for(h->pitch);
    auto bail = [&](int code) {
        sw2d_destroy(h);
        return code;
    };
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) return bail(SW2D_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(SW2D_ERR_CUDA);
    const size_t fb = h->plane * h->real_size;
    // allocate with the zero frame, keep pointers at cell (0,0)
    auto alloc_field = [&](void **p, size_t esz) -> bool {
        void *raw = nullptr;
        if (cudaMalloc(&raw, h->plane * esz) != cudaSuccess) return false;
        if (cudaMemset(raw, 0, h->plane * esz) != cudaSuccess) return false;
        *p = static_cast<char *>(raw) + h->origin * esz;
        return true;
    };
    for (int b = 0; b < 2; b++) {
        void **arrs[3] = {&h->h[b], &h->um[b], &h->vn[b]};
        for (void **a : arrs)
            if (!alloc_field(a, h->real_size)) return bail(SW2D_ERR_OOM);
    }
    if (!alloc_field(&h->z, h->real_size) || !alloc_field(&h->nman, h->real_size) ||
        !alloc_field((void **)&h->mask, 1))
        return bail(SW2D_ERR_OOM);
    (void)fb;
    h->stage_elems = (size_t)(cfg->rows + 1) * (cfg->cols + 1);
    if (cudaMalloc((void **)&h->stage, h->stage_elems * sizeof(double)) != cudaSuccess) return bail(SW2D_ERR_OOM);
    if (cudaMalloc((void **)&h->stage2, h->stage_elems * sizeof(double)) != cudaSuccess) return bail(SW2D_ERR_OOM);
    if (cudaMalloc((void **)&h->partial, kVolumeBlocks * sizeof(double)) != cudaSuccess) return bail(SW2D_ERR_OOM);
    if (cudaMalloc((void **)&h->d_clk, 3 * sizeof(Clock)) != cudaSuccess) return bail(SW2D_ERR_OOM);
    if (cudaMalloc((void **)&h->d_ctl, sizeof(Control)) != cudaSuccess) return bail(SW2D_ERR_OOM);
    if (cudaMallocHost((void **)&h->h_clk, sizeof(Clock)) != cudaSuccess) return bail(SW2D_ERR_OOM);
    if (cudaMallocHost((void **)&h->h_ctl, sizeof(Control)) != cudaSuccess) return bail(SW2D_ERR_OOM);
    if (cudaMallocHost((void **)&h->h_partial, kVolumeBlocks * sizeof(double)) != cudaSuccess) return bail(SW2D_ERR_OOM);
    if (cudaMemset(h->d_clk, 0, 3 * sizeof(Clock)) != cudaSuccess) return bail(SW2D_ERR_CUDA);
    h->stream_kernel = cfg->precision == SW2D_PREC_F32 && cfg->kernel != SW2D_KERNEL_TILE;
    h->variant = cfg->variant;
    if (h->stream_kernel && (!alloc_field(&h->dzx, h->real_size) || !alloc_field(&h->dzy, h->real_size) ||
                             !alloc_field(&h->hr[0], h->real_size) || !alloc_field(&h->hr[1], h->real_size)))
        return bail(SW2D_ERR_OOM);
    if (h->stream_kernel) {
        e = prepare_stream_step(h->variant);
    } else {
        e = is_f64(h) ? prepare_step(h->tile_h, h->tile_w, 0.0) : prepare_step(h->tile_h, h->tile_w, 0.0f);
    }
    if (e != cudaSuccess) return bail(SW2D_ERR_CUDA);

    GridDesc &G = h->G;
    G.rows = cfg->rows;
    G.cols = cfg->cols;
    G.pitch = h->pitch;
    G.tiles_w = (cfg->cols + h->tile_w - 1) / h->tile_w;
    const int tiles_h = (cfg->rows + h->tile_h - 1) / h->tile_h;
    h->nblocks = tiles_h * G.tiles_w;
    if (h->stream_kernel) {
        const int oc = stream_out_cols();
        h->stream_tiles_w = (cfg->cols + oc - 1) / oc;
        const int nw = stream_warps(h->variant);
        int sh = cfg->strip_h;
        // several iterations per launch under the fixed time step, when every
        // unit fits one wave of resident warps (asked for: an error otherwise)
        if (cfg->dt_mode == SW2D_DT_FIXED && cfg->steps_per_launch != 1) {
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg->device);
            const long long resident = (long long)sms * stream_pipe_ctas_per_sm(h->variant) * nw;
            const int psh = sh > 0 ? sh : pipe_strip(cfg->rows, h->stream_tiles_w, resident);
            const long long strips = psh > 0 ? (cfg->rows + psh - 1) / psh : 0;
            const long long units = (long long)h->stream_tiles_w * strips;
            // strips split the rows evenly: the shortest has rows / strips rows
            const bool tall = strips == 1 || (strips > 1 && cfg->rows / strips >= stream_pipe_min_strip());
            // the library's choice: pipelined where one wave holds the grid in
            // short strips (measured on GB300: 1.12-1.30x faster than one launch
            // per iteration up to 1024^2, whose iterations are mostly the
            // grid-wide drain; about even with 52-row strips at 2048^2, slower
            // with the long strips one wave needs beyond)
            const bool worth = cfg->steps_per_launch > 1 || psh <= kAutoPipeMaxStrip;
            if (tall && worth && units > 0 && units <= resident) {
                h->pipe_k = cfg->steps_per_launch > 1 ? cfg->steps_per_launch : kChunk;
                h->pipe_auto = cfg->steps_per_launch == 0;
                sh = psh;
            } else if (cfg->steps_per_launch > 1) {
                h->err = "steps_per_launch > 1: the units must fit one wave of resident warps, in strips of at least 8 rows";
                return bail(SW2D_ERR_INVALID_ARG);
            }
        }
        if (sh <= 0) sh = auto_strip(cfg->rows, h->stream_tiles_w, h->variant, cfg->device);
        h->strip_h = sh;
        h->stream_units = h->stream_tiles_w * ((cfg->rows + sh - 1) / sh);
        h->nblocks = (h->stream_units + nw - 1) / nw;
        if (h->pipe_k == 0) {
            // one launch per iteration filling one wave of resident warps: the
            // warp scheduler favours the CTAs launched first, so their strips
            // get more rows (measured at 2048^2: 79.4 against 80.7 us)
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg->device);
            const long long resident = (long long)sms * stream_ctas_per_sm(h->variant) * nw;
            const int strips = (cfg->rows + sh - 1) / sh;
            if (h->stream_units <= resident && 10LL * h->stream_units >= 9 * resident && cfg->rows / strips >= 16)
                h->strip_skew = kStripSkew;
        }
        if (h->pipe_k > 0 && (cudaMalloc((void **)&h->d_plans, (size_t)h->pipe_k * sizeof(Plan)) != cudaSuccess ||
                              cudaMalloc((void **)&h->d_words, 2 * sizeof(unsigned)) != cudaSuccess ||
                              cudaMalloc((void **)&h->d_flags, 2 * (size_t)h->stream_units * sizeof(unsigned)) != cudaSuccess))
            return bail(SW2D_ERR_OOM);
    }
    G.dt_mode = cfg->dt_mode;
    G.south_open = cfg->south_open ? 1 : 0;
    G.n_src = 0;
    G.dx = cfg->dx;
    G.dy = cfg->dy;
    G.g = cfg->g;
    G.th = cfg->th;
    G.cfl = cfg->cfl;
    G.dmin = cfg->dx < cfg->dy ? cfg->dx : cfg->dy;
    G.dt_half = cfg->dt;
    G.sd.dx = cfg->dx;
    G.sd.dy = cfg->dy;
    G.sd.g = cfg->g;
    G.sd.manning = cfg->manning;
    G.sd.pct_hi = 1.00 - cfg->LWL;               // cu:628
    G.sd.pct_lo = 1.00 - (cfg->INT + cfg->INF);  // cu:632
    G.sd.storm_amp = 0.0;
    G.sd.storm_2s2 = 1.0;
    sync_grid_scalars(G);
    h->F.rain_kind = RAIN_NONE;
    h->F.rain_dt = 1.0;
    h->F.ev_dt = 1.0;
    h->F.dtoq = 1.0;
    *out = h;
    return SW2D_OK;
}

int sw2d_destroy(sw2d_handle *h) {
    if (!h) return SW2D_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    auto free_field = [&](void *p, size_t esz) {
        if (p) cudaFree(static_cast<char *>(p) - h->origin * esz);
    };
    for (int b = 0; b < 2; b++) {
        free_field(h->h[b], h->real_size);
        free_field(h->um[b], h->real_size);
        free_field(h->vn[b], h->real_size);
    }
    free_field(h->z, h->real_size);
    free_field(h->nman, h->real_size);
    free_field(h->mask, 1);
    free_field(h->rainw, h->real_size);
    free_field(h->dzx, h->real_size);
    free_field(h->hr[0], h->real_size);
    free_field(h->hr[1], h->real_size);
    free_field(h->dzy, h->real_size);
    cudaFree(h->stage);
    cudaFree(h->stage2);
    cudaFree(h->partial);
    cudaFree(h->d_clk);
    cudaFree(h->d_ctl);
    cudaFree(h->d_plans);
    cudaFree(h->d_words);
    cudaFree(h->d_flags);
    for (DevBuf *b : {&h->rain, &h->ev, &h->src_cell, &h->src_q, &h->probe_cells, &h->probe_out}) cudaFree(b->p);
    if (h->h_clk) cudaFreeHost(h->h_clk);
    if (h->h_ctl) cudaFreeHost(h->h_ctl);
    if (h->h_partial) cudaFreeHost(h->h_partial);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SW2D_OK;
}

int sw2d_set_static(sw2d_handle *h, const double *z, const double *manning) {
    if (!h || !z) return fail(h, SW2D_ERR_INVALID_ARG, "z is null");
    const int rows = h->cfg.rows, cols = h->cfg.cols;
    const size_t n = (size_t)rows * cols;
    CK(h, cudaMemcpyAsync(h->stage, z, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    double *dn = nullptr;
    if (manning) {
        CK(h, cudaMemcpyAsync(h->stage2, manning, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        dn = h->stage2;
    }
    if (is_f64(h))
        CK(h, launch_pack_static(h->stage, dn, rows, cols, h->pitch, h->cfg.nodata, (double *)h->z,
                                 dn ? (double *)h->nman : nullptr, h->mask, h->stream));
    else
        CK(h, launch_pack_static(h->stage, dn, rows, cols, h->pitch, h->cfg.nodata, (float *)h->z,
                                 dn ? (float *)h->nman : nullptr, h->mask, h->stream));
    if (h->stream_kernel)
        CK(h, launch_pack_dz(h->stage, rows, cols, h->pitch, h->mask, (float *)h->dzx, (float *)h->dzy, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->has_nraster = manning != nullptr;
    h->have_static = true;
    h->have_state = false;  // the active mask may have changed
    h->use_rainw = false;   // rain factors were packed with the old mask
    h->graph_valid = false;
    return SW2D_OK;
}

int sw2d_set_rain_weights(sw2d_handle *h, const double *w) {
    if (!h) return SW2D_ERR_INVALID_ARG;
    if (!h->have_static) return fail(h, SW2D_ERR_STATE, "sw2d_set_rain_weights needs sw2d_set_static first");
    h->graph_valid = false;
    if (!w) {
        h->use_rainw = false;
        return SW2D_OK;
    }
    const int rows = h->cfg.rows, cols = h->cfg.cols;
    const size_t n = (size_t)rows * cols;
    for (size_t k = 0; k < n; k++)
        if (!(w[k] >= 0.0) || !std::isfinite(w[k]))
            return fail(h, SW2D_ERR_INVALID_ARG, "rain weights must be finite and >= 0");
    if (!h->rainw) {
        void *p = nullptr;
        const size_t bytes = h->plane * h->real_size;
        CK(h, cudaMalloc(&p, bytes));
        CK(h, cudaMemsetAsync(p, 0, bytes, h->stream));  // zero frame
        h->rainw = static_cast<char *>(p) + h->origin * h->real_size;
    }
    CK(h, cudaMemcpyAsync(h->stage, w, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (is_f64(h))
        CK(h, launch_pack_depth(h->stage, rows, cols, h->pitch, h->mask, (double *)h->rainw, h->stream));
    else
        CK(h, launch_pack_depth(h->stage, rows, cols, h->pitch, h->mask, (float *)h->rainw, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->use_rainw = true;
    return SW2D_OK;
}

int sw2d_set_state(sw2d_handle *h, const double *depth, const double *um, const double *vn, double t0) {
    if (!h || !depth) return fail(h, SW2D_ERR_INVALID_ARG, "depth is null");
    if (!h->have_static) return fail(h, SW2D_ERR_STATE, "sw2d_set_static must come first");
    const int rows = h->cfg.rows, cols = h->cfg.cols, pitch = h->pitch;
    const size_t fb = h->plane * h->real_size;
    for (int b = 0; b < 2; b++) {
        CK(h, cudaMemsetAsync(raw_field(h, h->h[b]), 0, fb, h->stream));
        CK(h, cudaMemsetAsync(raw_field(h, h->um[b]), 0, fb, h->stream));
        CK(h, cudaMemsetAsync(raw_field(h, h->vn[b]), 0, fb, h->stream));
        if (h->hr[b]) CK(h, cudaMemsetAsync(raw_field(h, h->hr[b]), 0, fb, h->stream));
    }
    CK(h, cudaMemcpyAsync(h->stage, depth, (size_t)rows * cols * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (is_f64(h)) CK(h, launch_pack_depth(h->stage, rows, cols, pitch, h->mask, (double *)h->h[0], h->stream));
    else CK(h, launch_pack_depth(h->stage, rows, cols, pitch, h->mask, (float *)h->h[0], h->stream));
    const double *su = nullptr, *sv = nullptr;
    if (um) {
        CK(h, cudaMemcpyAsync(h->stage, um, (size_t)(rows + 1) * cols * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        su = h->stage;
    }
    if (is_f64(h)) CK(h, launch_pack_um(su, rows, cols, pitch, h->G.south_open, h->mask, (double *)h->um[0], h->stream));
    else CK(h, launch_pack_um(su, rows, cols, pitch, h->G.south_open, h->mask, (float *)h->um[0], h->stream));
    if (vn) {
        CK(h, cudaMemcpyAsync(h->stage2, vn, (size_t)rows * (cols + 1) * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        sv = h->stage2;
    }
    if (is_f64(h)) CK(h, launch_pack_vn(sv, rows, cols, pitch, h->mask, (double *)h->vn[0], h->stream));
    else CK(h, launch_pack_vn(sv, rows, cols, pitch, h->mask, (float *)h->vn[0], h->stream));
    // clock slot 0 = this state; slots 1 and 2 start with empty accumulators
    Clock c0{};
    c0.t = t0;
    c0.buf = 0;
    CK(h, cudaMemsetAsync(h->d_clk, 0, 3 * sizeof(Clock), h->stream));
    *h->h_clk = c0;
    CK(h, cudaMemcpyAsync(h->d_clk, h->h_clk, sizeof(Clock), cudaMemcpyHostToDevice, h->stream));
    if (is_f64(h))
        CK(h, launch_cmax((const double *)h->h[0], (const double *)h->um[0], (const double *)h->vn[0], h->mask, rows,
                          cols, pitch, h->G.south_open, make_thr<double>(h->cfg).ge_th, h->cfg.g,
                          &h->d_clk[0].cmax_bits, h->stream));
    else
        CK(h, launch_cmax((const float *)h->h[0], (const float *)h->um[0], (const float *)h->vn[0], h->mask, rows,
                          cols, pitch, h->G.south_open, make_thr<float>(h->cfg).ge_th, h->cfg.g,
                          &h->d_clk[0].cmax_bits, h->stream));
    h->launches = 0;
    h->kernels = 0;
    h->fold_needed = false;
    h->have_state = true;
    int rc = read_clock(h);
    if (rc) return rc;
    sw2d_budget b;
    rc = sw2d_get_budget(h, &b);
    if (rc) return rc;
    h->volume0 = b.volume;
    return SW2D_OK;
}

int sw2d_set_rain(sw2d_handle *h, int32_t kind, const double *series, int32_t n, double dt_series) {
    if (!h) return SW2D_ERR_INVALID_ARG;
    if (kind == SW2D_RAIN_NONE) {
        h->F.rain_kind = RAIN_NONE;
        h->graph_valid = false;
        return SW2D_OK;
    }
    if (kind != SW2D_RAIN_COMPAT && kind != SW2D_RAIN_STEP && kind != SW2D_RAIN_LINEAR)
        return fail(h, SW2D_ERR_INVALID_ARG, "rain kind must be NONE, COMPAT, STEP or LINEAR (storm: sw2d_set_storm)");
    if (!series || n < 1 || !(dt_series > 0)) return fail(h, SW2D_ERR_INVALID_ARG, "bad rain series");
    int rc = upload_table(h, h->rain, series, (size_t)n);
    if (rc) return rc;
    h->F.rain_kind = kind;
    h->F.rain = (const double *)h->rain.p;
    h->F.n_rain = n;
    h->F.rain_dt = dt_series;
    h->graph_valid = false;
    return SW2D_OK;
}

int sw2d_set_storm(sw2d_handle *h, double peak, double x0, double y0, double vx, double vy, double sigma,
                   double t_stop) {
    if (!h) return SW2D_ERR_INVALID_ARG;
    if (!(sigma > 0) || !(peak >= 0)) return fail(h, SW2D_ERR_INVALID_ARG, "storm needs sigma > 0 and peak >= 0");
    h->F.rain_kind = RAIN_STORM;
    h->F.storm_peak = peak;
    h->F.storm_x0 = x0;
    h->F.storm_y0 = y0;
    h->F.storm_vx = vx;
    h->F.storm_vy = vy;
    h->F.storm_sigma = sigma;
    h->F.storm_tstop = t_stop;
    h->G.sd.storm_amp = peak / 3.6e6;                // mm/h -> m/s
    h->G.sd.storm_2s2 = 2.0 * (sigma * sigma);
    sync_grid_scalars(h->G);
    h->graph_valid = false;
    return SW2D_OK;
}

int sw2d_set_evaporation(sw2d_handle *h, const double *series, int32_t n, double dt_series) {
    if (!h) return SW2D_ERR_INVALID_ARG;
    if (n <= 0) {
        h->F.n_ev = 0;
        h->graph_valid = false;
        return SW2D_OK;
    }
    if (!series || !(dt_series > 0)) return fail(h, SW2D_ERR_INVALID_ARG, "bad evaporation series");
    int rc = upload_table(h, h->ev, series, (size_t)n);
    if (rc) return rc;
    h->F.ev = (const double *)h->ev.p;
    h->F.n_ev = n;
    h->F.ev_dt = dt_series;
    h->graph_valid = false;
    return SW2D_OK;
}

int sw2d_evaporation_series(const double *temperature, const double *radiation, int32_t n, double albedo,
                            double dtime, double *evap_mm) {
    if (n < 0 || (n > 0 && (!temperature || !radiation || !evap_mm)) || !(dtime > 0.0))
        return SW2D_ERR_INVALID_ARG;
    // energy-balance evaporation per record: net radiation, the ITS-90 water
    // density polynomial (5-40 C) and the latent heat of vaporisation of
    // Henderson-Sellers (1984), in the operation order of the reference
    // (cu:557-587); this unit is compiled without FMA contraction, so every
    // value rounds as there (and as in the reference built with --fmad=false)
    for (int32_t i = 0; i < n; i++) {
        const double t = temperature[i];
        const double rs = (1 - albedo) * radiation[i];  // net radiation
        const double pw = 999.85308 + 6.32693 * (0.01) * t - 8.523829 * (0.001) * t * t +
                          6.943248 * (0.00001) * t * t * t - 3.821216 * (0.0000001) * t * t * t * t;
        const double tk = t + 273.15;
        const double lv = ((tk / (tk - 33.91)) * (tk / (tk - 33.91))) * 1.91846 * 1000000;
        const double e = (rs / (lv * pw)) * dtime * 1000.0;  // mm per record interval
        evap_mm[i] = e < 0 ? 0 : e;
    }
    return SW2D_OK;
}

int sw2d_set_point_sources(sw2d_handle *h, const int32_t *cells, int32_t n_src, const double *q, int32_t n_rec,
                           double dtoq) {
    if (!h) return SW2D_ERR_INVALID_ARG;
    if (n_src <= 0) {
        h->G.n_src = 0;
        h->graph_valid = false;
        return SW2D_OK;
    }
    if (!cells || !q || n_rec < 1 || !(dtoq > 0)) return fail(h, SW2D_ERR_INVALID_ARG, "bad point-source table");
    const long long ncell = (long long)h->cfg.rows * h->cfg.cols;
    for (int s = 0; s < n_src; s++)
        if (cells[s] < 0 || cells[s] >= ncell) return fail(h, SW2D_ERR_INVALID_ARG, "source cell out of range");
    int rc = upload_table(h, h->src_cell, cells, (size_t)n_src);
    if (rc) return rc;
    rc = upload_table(h, h->src_q, q, (size_t)n_src * n_rec);
    if (rc) return rc;
    h->F.src_cell = (const int *)h->src_cell.p;
    h->F.src_q = (const double *)h->src_q.p;
    h->F.n_qrec = n_rec;
    h->F.dtoq = dtoq;
    h->G.n_src = n_src;
    h->graph_valid = false;
    return SW2D_OK;
}

int sw2d_advance(sw2d_handle *h, int64_t max_steps, double t_end, int64_t *steps_done) {
    if (steps_done) *steps_done = 0;
    if (!h) return SW2D_ERR_INVALID_ARG;
    if (!h->have_static || !h->have_state) return fail(h, SW2D_ERR_STATE, "set_static and set_state must come first");
    if (max_steps < 0) return fail(h, SW2D_ERR_INVALID_ARG, "max_steps < 0");
    if (std::isnan(t_end)) return fail(h, SW2D_ERR_INVALID_ARG, "t_end is NaN");
    CK(h, cudaSetDevice(h->cfg.device));
    const long long start = h->clock.steps;
    Control ctl;
    ctl.t_end = t_end;
    ctl.step_limit = start + max_steps;
    *h->h_ctl = ctl;
    CK(h, cudaMemcpyAsync(h->d_ctl, h->h_ctl, sizeof(Control), cudaMemcpyHostToDevice, h->stream));
    // plan the next launch under the new control and the current forcing
    plan_kernel<<<1, 32, 0, h->stream>>>(h->G, h->F, h->d_clk, h->d_ctl, (int)(h->launches % 3));
    CK(h, cudaGetLastError());
    h->kernels++;
    for (;;) {
        double dtn;
        double cmax;
        std::memcpy(&cmax, &h->clock.cmax_bits, sizeof(double));
        if (!decide_step(h->clock.t, cmax, h->clock.steps, ctl, h->G, &dtn)) break;
        const long long remaining = ctl.step_limit - h->clock.steps;
        if (pipe_now(h)) {
            // up to pipe_k iterations in one cooperative launch (the plan
            // kernel stops it at step_limit and t_end)
            CK(h, launch_stream_pipe(h->variant, h->nblocks, h->stream_tiles_w, h->strip_h, h->stream_units, h->G,
                                     h->F, make_bufs<float>(h), make_thr<float>(h->cfg), h->d_clk, h->d_ctl,
                                     (int)(h->launches % 3), h->d_plans, h->d_words, h->d_flags, h->pipe_k,
                                     h->stream));
            h->launches++;
            h->kernels += 2;
        } else if (remaining >= kChunk) {
            if (!h->graph_valid) {
                int rc = capture_graph(h);
                if (rc) return rc;
            }
            CK(h, cudaGraphLaunch(h->graph, h->stream));
            h->launches += kChunk;
            h->kernels += kChunk;
            h->fold_needed = h->stream_kernel;
        } else {
            const long long n = ((remaining + 2) / 3) * 3;
            for (long long m = 0; m < n; m++) {
                CK(h, launch_one(h, (int)((h->launches) % 3)));
                h->launches++;
                h->kernels++;
                h->fold_needed = h->stream_kernel;
            }
        }
        int rc = read_clock(h);
        if (rc) return rc;
        if (h->clock.nonfinite) {
            if (steps_done) *steps_done = h->clock.steps - start;
            return fail(h, SW2D_ERR_NONFINITE, "a non-finite depth or discharge was produced");
        }
        if (h->clock.status & ST_TOO_MANY_LOCAL_SOURCES)
            return fail(h, SW2D_ERR_INVALID_ARG, "more than 64 point sources fall in one tile");
        if (h->clock.status & ST_PIPE_TIMEOUT)
            return fail(h, SW2D_ERR_TIMEOUT, "a pipelined launch gave up waiting for a neighbouring unit");
        if (!h->clock.ran) break;
    }
    if (steps_done) *steps_done = h->clock.steps - start;
    return SW2D_OK;
}

int sw2d_get_field(sw2d_handle *h, int32_t field, double *out) {
    if (!h || !out) return fail(h, SW2D_ERR_INVALID_ARG, "null argument");
    if (!h->have_state && field != SW2D_FIELD_ELEVATION) return fail(h, SW2D_ERR_STATE, "no state");
    const int rows = h->cfg.rows, cols = h->cfg.cols, pitch = h->pitch;
    const int b = h->clock.buf;
    const bool f64 = is_f64(h);
    int nr = rows, nc = cols;
    const void *src = nullptr, *add = nullptr;
    switch (field) {
    case SW2D_FIELD_DEPTH: src = h->h[b]; add = h->hr[b]; break;
    case SW2D_FIELD_UM: src = h->um[b]; nr = rows + 1; break;
    case SW2D_FIELD_VN: src = h->vn[b]; nc = cols + 1; break;
    case SW2D_FIELD_ELEVATION: src = h->z; break;
    case SW2D_FIELD_UU:
    case SW2D_FIELD_VV: {
        if (f64)
            CK(h, launch_velocity((const double *)h->h[b], (const double *)h->um[b], (const double *)h->vn[b], rows, cols,
                                  pitch, make_thr<double>(h->cfg).ge_th, h->stage, h->stage2, h->stream));
        else
            CK(h, launch_velocity((const float *)h->h[b], (const float *)h->um[b], (const float *)h->vn[b], rows, cols,
                                  pitch, make_thr<float>(h->cfg).ge_th, h->stage, h->stage2, h->stream));
        const double *s = field == SW2D_FIELD_UU ? h->stage : h->stage2;
        CK(h, cudaMemcpyAsync(out, s, (size_t)rows * cols * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        return SW2D_OK;
    }
    default:
        return fail(h, SW2D_ERR_INVALID_ARG, "unknown field");
    }
    if (f64) CK(h, launch_unpack((const double *)src, (const double *)add, nr, nc, pitch, h->stage, h->stream));
    else CK(h, launch_unpack((const float *)src, (const float *)add, nr, nc, pitch, h->stage, h->stream));
    CK(h, cudaMemcpyAsync(out, h->stage, (size_t)nr * nc * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return SW2D_OK;
}

int sw2d_get_budget(sw2d_handle *h, sw2d_budget *out) {
    if (!h || !out) return fail(h, SW2D_ERR_INVALID_ARG, "null argument");
    if (!h->have_state) return fail(h, SW2D_ERR_STATE, "no state");
    const int b = h->clock.buf;
    if (is_f64(h))
        CK(h, launch_volume((const double *)h->h[b], nullptr, h->mask, h->cfg.rows, h->cfg.cols, h->pitch,
                            h->partial, kVolumeBlocks, h->stream));
    else
        CK(h, launch_volume((const float *)h->h[b], (const float *)h->hr[b], h->mask, h->cfg.rows, h->cfg.cols,
                            h->pitch, h->partial, kVolumeBlocks, h->stream));
    CK(h, cudaMemcpyAsync(h->h_partial, h->partial, kVolumeBlocks * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    double s = 0.0, c = 0.0;
    for (int k = 0; k < kVolumeBlocks; k++) {
        double y = h->h_partial[k] - c;
        double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    const Clock &k = h->clock;
    double tot[B_N];
    for (int q = 0; q < B_N; q++) {  // fold the last iteration's sums
        double y = k.step[q] - k.tot_c[q];
        tot[q] = k.tot_s[q] + y;
    }
    std::memset(out, 0, sizeof(*out));
    out->t = k.t;
    out->dt = k.dt;
    std::memcpy(&out->cmax, &k.cmax_bits, sizeof(double));
    out->volume = s * h->cfg.dx * h->cfg.dy;
    out->volume0 = h->volume0;
    out->rain_in = tot[B_RAIN];
    out->source_in = tot[B_SRC];
    out->evap_out = tot[B_EV];
    out->outflow = tot[B_OUT];
    out->clamp_gain = tot[B_CLAMP];
    out->steps = k.steps;
    out->nonfinite = k.nonfinite ? 1 : 0;
    return SW2D_OK;
}

int sw2d_probe(sw2d_handle *h, const int32_t *cells, int32_t n, double *out) {
    if (!h || (n > 0 && (!cells || !out))) return fail(h, SW2D_ERR_INVALID_ARG, "null argument");
    if (!h->have_state) return fail(h, SW2D_ERR_STATE, "no state");
    if (n <= 0) return SW2D_OK;
    const long long ncell = (long long)h->cfg.rows * h->cfg.cols;
    for (int s = 0; s < n; s++)
        if (cells[s] < 0 || cells[s] >= ncell) return fail(h, SW2D_ERR_INVALID_ARG, "probe cell out of range");
    int rc = upload_table(h, h->probe_cells, cells, (size_t)n);
    if (rc) return rc;
    if (h->probe_out.bytes < (size_t)n * sizeof(double)) {
        cudaFree(h->probe_out.p);
        h->probe_out.p = nullptr;
        h->probe_out.bytes = 0;
        CK(h, cudaMalloc(&h->probe_out.p, (size_t)n * sizeof(double)));
        h->probe_out.bytes = (size_t)n * sizeof(double);
    }
    const int b = h->clock.buf;
    if (is_f64(h))
        CK(h, launch_probe((const double *)h->h[b], nullptr, h->cfg.rows, h->cfg.cols, h->pitch,
                           (const int *)h->probe_cells.p, n, (double *)h->probe_out.p, h->stream));
    else
        CK(h, launch_probe((const float *)h->h[b], (const float *)h->hr[b], h->cfg.rows, h->cfg.cols, h->pitch,
                           (const int *)h->probe_cells.p, n, (double *)h->probe_out.p, h->stream));
    CK(h, cudaMemcpyAsync(out, h->probe_out.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return SW2D_OK;
}

namespace {
struct CheckpointHeader {
    char magic[8];  // "SW2DCKP1"
    int32_t rows, cols, pitch, precision;
    int32_t nplanes, pad;  // h, um, vn (+ the depth remainder of the compensated FP32 state)
    int64_t plane_bytes;
    double volume0;
    Clock clock;
};
int checkpoint_planes(const sw2d_handle *h) { return h->hr[0] ? 4 : 3; }
}  // namespace

int sw2d_checkpoint_bytes(sw2d_handle *h, int64_t *bytes) {
    if (!h || !bytes) return SW2D_ERR_INVALID_ARG;
    *bytes = (int64_t)(sizeof(CheckpointHeader) + checkpoint_planes(h) * h->plane * h->real_size);
    return SW2D_OK;
}

int sw2d_checkpoint_save(sw2d_handle *h, void *buf, int64_t bytes) {
    int64_t need = 0;
    if (!h || !buf) return fail(h, SW2D_ERR_INVALID_ARG, "null argument");
    sw2d_checkpoint_bytes(h, &need);
    if (bytes < need) return fail(h, SW2D_ERR_INVALID_ARG, "checkpoint buffer too small");
    if (!h->have_state) return fail(h, SW2D_ERR_STATE, "no state");
    int rc = read_clock(h);
    if (rc) return rc;
    CheckpointHeader hd;
    std::memset(&hd, 0, sizeof(hd));
    std::memcpy(hd.magic, "SW2DCKP1", 8);
    hd.rows = h->cfg.rows;
    hd.cols = h->cfg.cols;
    hd.pitch = h->pitch;
    hd.precision = h->cfg.precision;
    hd.plane_bytes = (int64_t)(h->plane * h->real_size);
    hd.nplanes = checkpoint_planes(h);
    hd.volume0 = h->volume0;
    hd.clock = h->clock;
    char *p = static_cast<char *>(buf);
    std::memcpy(p, &hd, sizeof(hd));
    p += sizeof(hd);
    const int b = h->clock.buf;
    void *src[4] = {raw_field(h, h->h[b]), raw_field(h, h->um[b]), raw_field(h, h->vn[b]),
                    h->hr[b] ? raw_field(h, h->hr[b]) : nullptr};
    for (int k = 0; k < hd.nplanes; k++) {
        CK(h, cudaMemcpyAsync(p, src[k], (size_t)hd.plane_bytes, cudaMemcpyDeviceToHost, h->stream));
        p += hd.plane_bytes;
    }
    CK(h, cudaStreamSynchronize(h->stream));
    return SW2D_OK;
}

int sw2d_checkpoint_load(sw2d_handle *h, const void *buf, int64_t bytes) {
    if (!h || !buf) return fail(h, SW2D_ERR_INVALID_ARG, "null argument");
    if (!h->have_static) return fail(h, SW2D_ERR_STATE, "sw2d_set_static must come first");
    if (bytes < (int64_t)sizeof(CheckpointHeader)) return fail(h, SW2D_ERR_INVALID_ARG, "not a checkpoint");
    CheckpointHeader hd;
    std::memcpy(&hd, buf, sizeof(hd));
    int64_t need = 0;
    sw2d_checkpoint_bytes(h, &need);
    if (std::memcmp(hd.magic, "SW2DCKP1", 8) != 0 || hd.rows != h->cfg.rows || hd.cols != h->cfg.cols ||
        hd.pitch != h->pitch || hd.precision != h->cfg.precision || hd.nplanes != checkpoint_planes(h) ||
        bytes < need)
        return fail(h, SW2D_ERR_INVALID_ARG, "checkpoint does not match this handle's config");
    const char *p = static_cast<const char *>(buf) + sizeof(hd);
    void *dst[4] = {raw_field(h, h->h[0]), raw_field(h, h->um[0]), raw_field(h, h->vn[0]),
                    h->hr[0] ? raw_field(h, h->hr[0]) : nullptr};
    for (int k = 0; k < hd.nplanes; k++) {
        CK(h, cudaMemcpyAsync(dst[k], p, (size_t)hd.plane_bytes, cudaMemcpyHostToDevice, h->stream));
        p += hd.plane_bytes;
    }
    const size_t fb = h->plane * h->real_size;
    CK(h, cudaMemsetAsync(raw_field(h, h->h[1]), 0, fb, h->stream));
    CK(h, cudaMemsetAsync(raw_field(h, h->um[1]), 0, fb, h->stream));
    CK(h, cudaMemsetAsync(raw_field(h, h->vn[1]), 0, fb, h->stream));
    if (h->hr[1]) CK(h, cudaMemsetAsync(raw_field(h, h->hr[1]), 0, fb, h->stream));
    // the saved clock becomes slot 0 of a fresh launch sequence
    Clock c = hd.clock;
    c.buf = 0;
    c.cmax_bits = hd.clock.cmax_bits;
    c.done_blocks = 0;
    for (int q = 0; q < B_N; q++)
        for (int bb = 0; bb < kBuckets; bb++) c.stepb[q][bb] = 0.0;
    for (int bb = 0; bb < kBuckets; bb++) c.cmaxb[bb] = 0ull;
    CK(h, cudaMemsetAsync(h->d_clk, 0, 3 * sizeof(Clock), h->stream));
    *h->h_clk = c;
    CK(h, cudaMemcpyAsync(h->d_clk, h->h_clk, sizeof(Clock), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->launches = 0;
    h->kernels = 0;
    h->fold_needed = false;
    h->clock = c;
    h->volume0 = hd.volume0;
    h->have_state = true;
    return SW2D_OK;
}

int sw2d_synchronize(sw2d_handle *h) {
    if (!h) return SW2D_ERR_INVALID_ARG;
    CK(h, cudaStreamSynchronize(h->stream));
    return SW2D_OK;
}

int sw2d_get_stream(sw2d_handle *h, void **stream) {
    if (!h || !stream) return SW2D_ERR_INVALID_ARG;
    *stream = (void *)h->stream;
    return SW2D_OK;
}

int sw2d_launch_count(sw2d_handle *h, int64_t *launches) {
    if (!h || !launches) return SW2D_ERR_INVALID_ARG;
    *launches = h->kernels;
    return SW2D_OK;
}

int sw2d_describe(const sw2d_handle *h, char *buf, int32_t n) {
    if (!h || !buf || n <= 0) return SW2D_ERR_INVALID_ARG;
    if (h->stream_kernel) {
        // the forcing build the launcher picks (step_f32.cu): storm and point
        // sources, per-cell rain factors, or neither
        const bool gen = h->F.rain_kind == RAIN_STORM || h->G.n_src > 0;
        if (pipe_now(h))
            snprintf(buf, (size_t)n, "stream_pipe_kernel%s forcing=%s%s strip_h=%d units=%d ctas=%d steps_per_launch=%d",
                     std::strchr(stream_variant_name(h->variant), '<'), gen ? "storm/sources" : "uniform",
                     h->use_rainw ? "+rain_weights" : "", h->strip_h, h->stream_units, h->nblocks, h->pipe_k);
        else {
            char skew_s[32] = "";
            if (h->strip_skew) snprintf(skew_s, sizeof(skew_s), " strip_skew=%d", h->strip_skew);
            snprintf(buf, (size_t)n, "%s forcing=%s%s strip_h=%d units=%d ctas=%d steps_per_launch=1%s",
                     stream_variant_name(h->variant), gen ? "storm/sources" : "uniform",
                     h->use_rainw ? "+rain_weights" : "", h->strip_h, h->stream_units, h->nblocks, skew_s);
        }
    }
    else
        snprintf(buf, (size_t)n, "step_kernel<%s,%d,%d> ctas=%d", is_f64(h) ? "double" : "float", h->tile_h,
                 h->tile_w, h->nblocks);
    return SW2D_OK;
}

const char *sw2d_last_error(const sw2d_handle *h) { return h ? h->err.c_str() : "null handle"; }

const char *sw2d_status_string(int32_t s) {
    switch (s) {
    case SW2D_OK: return "ok";
    case SW2D_ERR_INVALID_ARG: return "invalid argument";
    case SW2D_ERR_OOM: return "out of device memory";
    case SW2D_ERR_CUDA: return "CUDA error";
    case SW2D_ERR_NONFINITE: return "non-finite value produced";
    case SW2D_ERR_TIMEOUT: return "device-side wait timed out";
    case SW2D_ERR_STATE: return "call order";
    default: return "unknown status";
    }
}

}  // extern "C"
