// sw2d_batch.cu -- host side of the batched FP32 solver (C ABI in
// include/sw2d.h, sw2d_batch_*).
//
// A batch owns one stream, a table of scenario descriptors, the unit table,
// a status array and three CUDA graphs of `chunk` launches (one per launch
// parity, because the clock slots rotate with the launch count).  Scenario
// memory is allocated stream-ordered (cudaMallocAsync) when a scenario is
// admitted and released the same way when it is retired, so admission and
// retirement never stall the GPU.  Compiled with the same flags as the FP32
// single-scenario kernels, so a scenario advances bit for bit as it would in
// its own handle.
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sw2d.h"
#include "sw2d_batch.cuh"
#include "sw2d_launch.h"

using namespace sw2d;

namespace {

// Builds of the batched kernel the autotuner chooses from: (id, warps per
// CTA, minimum resident CTAs per SM -- the register budget --, unrolling of
// the row loop).  Build 0 is the default: 8 warps and 2 CTAs per SM leave
// room for the queue state without spilling.
#define SW2D_BATCH_VARIANTS(X) X(0, 8, 2, 1) X(1, 8, 2, 2) X(2, 4, 4, 1)
constexpr int kBatchVariants = 3;

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct HostScenario {
    bool active = false;
    sw2d_config cfg{};
    int pitch = 0, tiles_w = 0, strip_h = 0, nunits = 0;
    bool raster = false;
    void *block = nullptr;
    size_t bytes = 0;
    double volume0 = 0.0;  // water of the admitted state [m^3]
    ScenarioDev dev{};
};

}  // namespace

struct sw2d_batch {
    sw2d_batch_config cfg{};
    cudaStream_t stream = nullptr;
    ScenarioDev *d_scen = nullptr;
    int2 *d_units = nullptr;
    BatchHeader *d_hdr = nullptr;
    ScenarioStatus *d_status = nullptr;
    ScenarioStatus *h_status = nullptr;  // pinned
    double *d_stage = nullptr;
    size_t stage_elems = 0;
    double *d_partial = nullptr;
    double *h_partial = nullptr;  // pinned
    Clock *h_clk = nullptr;       // pinned
    std::vector<HostScenario> scen;
    std::vector<int2> units;
    long long launches = 0;
    int grid = 0;
    cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
    int64_t bytes_in_use = 0;
    std::string err;
};

namespace {

int bfail(sw2d_batch *b, int code, const std::string &m) {
    if (b) b->err = m;
    return code;
}

#define BCK(b, expr)                                                                                 \
    do {                                                                                             \
        cudaError_t e_ = (expr);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return bfail((b), e_ == cudaErrorMemoryAllocation ? SW2D_ERR_OOM : SW2D_ERR_CUDA,        \
                         std::string(#expr) + ": " + cudaGetErrorString(e_));                         \
    } while (0)

cudaError_t launch_batch(sw2d_batch *b, int slot) {
    BatchDev B;
    B.scen = b->d_scen;
    B.units = b->d_units;
    B.hdr = b->d_hdr;
    // a programmatic dependent of the launch before it: its CTAs are
    // scheduled while that one drains, and wait for it to complete
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(b->grid);
    lc.dynamicSmemBytes = 0;
    lc.stream = b->stream;
    lc.attrs = attr;
    lc.numAttrs = 1;
#define SW2D_BL(id, nw, mb, un)                                                                 \
    if (b->cfg.variant == id) {                                                                 \
        lc.blockDim = dim3(nw * 32);                                                            \
        return cudaLaunchKernelEx(&lc, batch_step_kernel<nw, mb, un>, B, slot);                 \
    }
    SW2D_BATCH_VARIANTS(SW2D_BL)
#undef SW2D_BL
    return cudaErrorInvalidValue;
}

// Resident CTAs per SM of a build (its grid is that many per SM), 0 on error.
int batch_ctas_per_sm(int variant) {
    int n = 0;
#define SW2D_BO(id, nw, mb, un)                                                                              \
    if (variant == id &&                                                                                     \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_step_kernel<nw, mb, un>, nw * 32, 0) != cudaSuccess) \
        n = 0;
    SW2D_BATCH_VARIANTS(SW2D_BO)
#undef SW2D_BO
    return n;
}

int capture(sw2d_batch *b, int parity) {
    cudaGraph_t g = nullptr;
    BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int m = 0; m < b->cfg.chunk && e == cudaSuccess; m++) e = launch_batch(b, (parity + m) % 3);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(b, SW2D_ERR_CUDA, "batch graph capture failed");
    }
    e = cudaGraphInstantiate(&b->graph[parity], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, SW2D_ERR_CUDA, "batch graph instantiate failed");
    return SW2D_OK;
}

int upload_units(sw2d_batch *b) {
    b->units.clear();
    try {  // no exception crosses the C ABI
        for (size_t s = 0; s < b->scen.size(); s++) {
            const HostScenario &h = b->scen[s];
            if (!h.active) continue;
            for (int u = 0; u < h.nunits; u++) b->units.push_back(make_int2((int)s, u));
        }
    } catch (...) {
        return bfail(b, SW2D_ERR_OOM, "host memory for the unit table");
    }
    if ((long long)b->units.size() > b->cfg.max_units)
        return bfail(b, SW2D_ERR_INVALID_ARG, "unit table full: raise max_units");
    if (!b->units.empty())
        BCK(b, cudaMemcpyAsync(b->d_units, b->units.data(), b->units.size() * sizeof(int2), cudaMemcpyHostToDevice,
                               b->stream));
    const int n = (int)b->units.size();
    BCK(b, cudaMemcpyAsync(&b->d_hdr->n_units, &n, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));  // the host vector and n must outlive the copies
    return SW2D_OK;
}

// rows per warp: the scenario's own setting (autotuned), the batch's, or by size
int strip_for(const sw2d_batch *b, const sw2d_config *c) {
    if (c->strip_h > 0) return c->strip_h;
    if (b->cfg.strip_h > 0) return b->cfg.strip_h;
    return c->rows >= 1024 ? 64 : (c->rows >= 256 ? 32 : 16);
}

template <class T>
T *carve(char *base, size_t &off, size_t n) {
    T *p = reinterpret_cast<T *>(base + off);
    off += align256(n * sizeof(T));
    return p;
}

size_t scenario_bytes(const sw2d_config *c, int n_rain, bool raster) {
    const int pitch = pitch_for(c->cols);
    const size_t plane = plane_for(c->rows, pitch);
    size_t s = 0;
    s += 8 * align256(plane * sizeof(float));                    // h, um, vn, depth remainder x 2
    s += 3 * align256(plane * sizeof(float));                    // z, dzx, dzy
    if (raster) s += align256(plane * sizeof(float));            // n
    s += align256(plane);                                        // mask
    s += align256(3 * sizeof(Clock));                            // clock slots
    s += align256((size_t)(n_rain > 0 ? n_rain : 1) * sizeof(double));
    return s;
}

}  // namespace

extern "C" {

int sw2d_batch_config_init(sw2d_batch_config *c) {
    if (!c) return SW2D_ERR_INVALID_ARG;
    std::memset(c, 0, sizeof(*c));
    c->device = 0;
    c->max_scenarios = 1024;
    c->max_units = 1 << 20;
    c->strip_h = 0;
    c->max_bytes = 0;
    c->chunk = 24;
    return SW2D_OK;
}

int sw2d_batch_scenario_bytes(const sw2d_config *cfg, int32_t n_rain, int32_t with_raster, int64_t *bytes) {
    if (!cfg || !bytes || !plane_fits_int32(cfg->rows, cfg->cols) || n_rain < 0) return SW2D_ERR_INVALID_ARG;
    *bytes = (int64_t)scenario_bytes(cfg, n_rain, with_raster != 0);
    return SW2D_OK;
}

int sw2d_batch_create(const sw2d_batch_config *cfg, sw2d_batch **out) {
    if (!cfg || !out) return SW2D_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->max_scenarios < 1 || cfg->max_units < 1 || cfg->chunk < 3 || cfg->chunk % 3 != 0 || cfg->strip_h < 0 ||
        cfg->variant < 0 || cfg->variant >= kBatchVariants)
        return SW2D_ERR_INVALID_ARG;
    sw2d_batch *b = new (std::nothrow) sw2d_batch();  // no exception crosses the C ABI
    if (!b) return SW2D_ERR_OOM;
    b->cfg = *cfg;
    auto bail = [&](int code) {
        sw2d_batch_destroy(b);
        return code;
    };
    if (cudaSetDevice(cfg->device) != cudaSuccess) return bail(SW2D_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(SW2D_ERR_CUDA);
    if (cudaMalloc((void **)&b->d_scen, (size_t)cfg->max_scenarios * sizeof(ScenarioDev)) != cudaSuccess ||
        cudaMalloc((void **)&b->d_units, (size_t)cfg->max_units * sizeof(int2)) != cudaSuccess ||
        cudaMalloc((void **)&b->d_hdr, sizeof(BatchHeader)) != cudaSuccess ||
        cudaMalloc((void **)&b->d_status, (size_t)cfg->max_scenarios * sizeof(ScenarioStatus)) != cudaSuccess ||
        cudaMalloc((void **)&b->d_partial, kVolumeBlocks * sizeof(double)) != cudaSuccess)
        return bail(SW2D_ERR_OOM);
    if (cudaMallocHost((void **)&b->h_status, (size_t)cfg->max_scenarios * sizeof(ScenarioStatus)) != cudaSuccess ||
        cudaMallocHost((void **)&b->h_partial, kVolumeBlocks * sizeof(double)) != cudaSuccess ||
        cudaMallocHost((void **)&b->h_clk, sizeof(Clock)) != cudaSuccess)
        return bail(SW2D_ERR_OOM);
    cudaMemset(b->d_hdr, 0, sizeof(BatchHeader));
    cudaMemset(b->d_scen, 0, (size_t)cfg->max_scenarios * sizeof(ScenarioDev));
    cudaMemset(b->d_status, 0, (size_t)cfg->max_scenarios * sizeof(ScenarioStatus));
    try {
        b->scen.resize(cfg->max_scenarios);
    } catch (...) {
        return bail(SW2D_ERR_OOM);
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg->device);
    int per_sm = batch_ctas_per_sm(cfg->variant);
    if (per_sm < 1) per_sm = 1;
    b->grid = (sms > 0 ? sms : 152) * per_sm;
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(SW2D_ERR_CUDA);
    *out = b;
    return SW2D_OK;
}

int sw2d_batch_destroy(sw2d_batch *b) {
    if (!b) return SW2D_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (int p = 0; p < 3; p++)
        if (b->graph[p]) cudaGraphExecDestroy(b->graph[p]);
    for (HostScenario &h : b->scen)
        if (h.block) cudaFree(h.block);
    cudaFree(b->d_scen);
    cudaFree(b->d_units);
    cudaFree(b->d_hdr);
    cudaFree(b->d_status);
    cudaFree(b->d_partial);
    cudaFree(b->d_stage);
    if (b->h_status) cudaFreeHost(b->h_status);
    if (b->h_partial) cudaFreeHost(b->h_partial);
    if (b->h_clk) cudaFreeHost(b->h_clk);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return SW2D_OK;
}

namespace {
// Water on the active cells of buffer `buf` of a scenario [m^3]: deterministic
// FP64 partials on the device (depth + remainder), Kahan-summed here; waits.
int scenario_volume(sw2d_batch *b, const HostScenario &h, int buf, double *vol) {
    BCK(b, launch_volume(h.dev.h[buf], h.dev.hr[buf], h.dev.mask, h.cfg.rows, h.cfg.cols, h.pitch, b->d_partial,
                         kVolumeBlocks, b->stream));
    BCK(b, cudaMemcpyAsync(b->h_partial, b->d_partial, kVolumeBlocks * sizeof(double), cudaMemcpyDeviceToHost,
                           b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    double s = 0.0, c = 0.0;
    for (int q = 0; q < kVolumeBlocks; q++) {
        const double y = b->h_partial[q] - c;
        const double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    *vol = s * h.cfg.dx * h.cfg.dy;
    return SW2D_OK;
}
}  // namespace

int sw2d_batch_add(sw2d_batch *b, const sw2d_config *cfg, const double *z, const double *manning,
                   const double *depth, int32_t rain_kind, const double *rain, int32_t n_rain, double rain_dt,
                   double t_end, int32_t *id) {
    if (!b || !cfg || !z || !depth || !id) return bfail(b, SW2D_ERR_INVALID_ARG, "null argument");
    if (cfg->precision != SW2D_PREC_F32 || cfg->dt_mode != SW2D_DT_CFL)
        return bfail(b, SW2D_ERR_INVALID_ARG, "batched scenarios are FP32 with the CFL rule");
    if (cfg->rows < 1 || cfg->cols < 1 || !(cfg->dx > 0) || !(cfg->dy > 0) || !(cfg->dt > 0) || !(cfg->cfl > 0))
        return bfail(b, SW2D_ERR_INVALID_ARG, "bad grid or time-step settings");
    if (!plane_fits_int32(cfg->rows, cfg->cols)) return bfail(b, SW2D_ERR_INVALID_ARG, "grid too large for 32-bit indexing");
    if (rain_kind != SW2D_RAIN_NONE && rain_kind != SW2D_RAIN_COMPAT && rain_kind != SW2D_RAIN_STEP &&
        rain_kind != SW2D_RAIN_LINEAR)
        return bfail(b, SW2D_ERR_INVALID_ARG, "rain kind");
    if (rain_kind != SW2D_RAIN_NONE && (!rain || n_rain < 1 || !(rain_dt > 0)))
        return bfail(b, SW2D_ERR_INVALID_ARG, "bad rain series");
    int slot = -1;
    for (int s = 0; s < (int)b->scen.size(); s++)
        if (!b->scen[s].active && b->scen[s].block == nullptr) {
            slot = s;
            break;
        }
    if (slot < 0) return bfail(b, SW2D_ERR_INVALID_ARG, "scenario table full: raise max_scenarios");
    const bool raster = manning != nullptr;
    const size_t need = scenario_bytes(cfg, rain_kind == SW2D_RAIN_NONE ? 0 : n_rain, raster);
    if (b->cfg.max_bytes > 0 && b->bytes_in_use + (int64_t)need > b->cfg.max_bytes)
        return bfail(b, SW2D_ERR_OOM, "batch memory budget exceeded");
    HostScenario &h = b->scen[slot];
    h = HostScenario();
    h.cfg = *cfg;
    h.raster = raster;
    h.pitch = pitch_for(cfg->cols);
    h.strip_h = strip_for(b, cfg);
    h.tiles_w = (cfg->cols + stream_out_cols() - 1) / stream_out_cols();
    h.nunits = h.tiles_w * ((cfg->rows + h.strip_h - 1) / h.strip_h);
    BCK(b, cudaSetDevice(b->cfg.device));
    BCK(b, cudaMallocAsync(&h.block, need, b->stream));
    h.bytes = need;
    b->bytes_in_use += (int64_t)need;
    const size_t plane = plane_for(cfg->rows, h.pitch), org = origin_for(h.pitch);
    char *base = static_cast<char *>(h.block);
    size_t off = 0;
    ScenarioDev &d = h.dev;
    std::memset(&d, 0, sizeof(d));
    // fields with their zero frame; pointers at cell (0,0)
    for (int k = 0; k < 2; k++) d.h[k] = carve<float>(base, off, plane) + org;
    for (int k = 0; k < 2; k++) d.um[k] = carve<float>(base, off, plane) + org;
    for (int k = 0; k < 2; k++) d.vn[k] = carve<float>(base, off, plane) + org;
    for (int k = 0; k < 2; k++) d.hr[k] = carve<float>(base, off, plane) + org;
    float *z_dev = carve<float>(base, off, plane) + org;
    float *dzx_dev = carve<float>(base, off, plane) + org;
    float *dzy_dev = carve<float>(base, off, plane) + org;
    float *n_dev = raster ? carve<float>(base, off, plane) + org : nullptr;
    uint8_t *m_dev = carve<uint8_t>(base, off, plane) + org;
    Clock *clk = carve<Clock>(base, off, 3);
    double *rain_dev = carve<double>(base, off, (size_t)(n_rain > 0 ? n_rain : 1));
    BCK(b, cudaMemsetAsync(h.block, 0, off, b->stream));
    // staging for the float64 host rasters
    const size_t cells = (size_t)cfg->rows * cfg->cols;
    if (b->stage_elems < 2 * cells) {
        if (b->d_stage) BCK(b, cudaFreeAsync(b->d_stage, b->stream));
        b->d_stage = nullptr;
        BCK(b, cudaMallocAsync((void **)&b->d_stage, 2 * cells * sizeof(double), b->stream));
        b->stage_elems = 2 * cells;
    }
    double *st0 = b->d_stage, *st1 = b->d_stage + cells;
    BCK(b, cudaMemcpyAsync(st0, z, cells * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    if (raster) BCK(b, cudaMemcpyAsync(st1, manning, cells * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    BCK(b, launch_pack_static(st0, raster ? st1 : nullptr, cfg->rows, cfg->cols, h.pitch, cfg->nodata, z_dev,
                              n_dev, m_dev, b->stream));
    BCK(b, launch_pack_dz(st0, cfg->rows, cfg->cols, h.pitch, m_dev, dzx_dev, dzy_dev, b->stream));
    BCK(b, cudaMemcpyAsync(st0, depth, cells * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    BCK(b, launch_pack_depth(st0, cfg->rows, cfg->cols, h.pitch, m_dev, d.h[0], b->stream));
    if (rain_kind != SW2D_RAIN_NONE)
        BCK(b, cudaMemcpyAsync(rain_dev, rain, (size_t)n_rain * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    // descriptor
    GridDesc &G = d.G;
    G.rows = cfg->rows;
    G.cols = cfg->cols;
    G.pitch = h.pitch;
    G.tiles_w = h.tiles_w;
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
    G.sd.rdx = 1.0 / cfg->dx;
    G.sd.rdy = 1.0 / cfg->dy;
    G.sd.pct_hi = 1.00 - cfg->LWL;
    G.sd.pct_lo = 1.00 - (cfg->INT + cfg->INF);
    G.sd.storm_amp = 0.0;
    G.sd.storm_2s2 = 1.0;
    G.sf.dx = (float)G.sd.dx;
    G.sf.dy = (float)G.sd.dy;
    G.sf.g = (float)G.sd.g;
    G.sf.manning = (float)G.sd.manning;
    G.sf.rdx = (float)G.sd.rdx;
    G.sf.rdy = (float)G.sd.rdy;
    G.sf.pct_hi = (float)G.sd.pct_hi;
    G.sf.pct_lo = (float)G.sd.pct_lo;
    G.sf.storm_amp = 0.f;
    G.sf.storm_2s2 = 1.f;
    ForcingDesc &F = d.F;
    F.rain_kind = rain_kind;
    F.rain = rain_dev;
    F.n_rain = rain_kind == SW2D_RAIN_NONE ? 0 : n_rain;
    F.rain_dt = rain_kind == SW2D_RAIN_NONE ? 1.0 : rain_dt;
    F.ev_dt = 1.0;
    F.dtoq = 1.0;
    {
        // thresholds, as the single-scenario FP32 path sets them
        float f = (float)cfg->th;
        if ((double)f < cfg->th) f = std::nextafter(f, INFINITY);
        d.T.ge_th = f;
        f = (float)cfg->th;
        if ((double)f <= cfg->th) f = std::nextafter(f, INFINITY);
        d.T.gt_th = f;
        f = (float)cfg->EV_WL_min;
        if ((double)f <= cfg->EV_WL_min) f = std::nextafter(f, INFINITY);
        d.T.gt_evmin = f;
    }
    d.ctl.t_end = t_end;
    d.ctl.step_limit = 1ll << 62;
    d.z = z_dev;
    d.dzx = dzx_dev;
    d.dzy = dzy_dev;
    d.nman = n_dev;
    d.mask = m_dev;
    d.clk = clk;
    int vrc = scenario_volume(b, h, 0, &h.volume0);  // the admitted state, as the FP32 planes hold it
    if (vrc) return vrc;
    d.status = b->d_status + slot;
    d.tiles_w = h.tiles_w;
    d.strip_h = h.strip_h;
    d.nunits = h.nunits;
    BCK(b, cudaMemcpyAsync(b->d_scen + slot, &d, sizeof(ScenarioDev), cudaMemcpyHostToDevice, b->stream));
    // clock: the current launch parity holds this state
    const int cur = (int)(b->launches % 3);
    Clock c0;
    std::memset(&c0, 0, sizeof(c0));
    *b->h_clk = c0;
    BCK(b, cudaMemcpyAsync(clk + cur, b->h_clk, sizeof(Clock), cudaMemcpyHostToDevice, b->stream));
    BCK(b, launch_cmax(d.h[0], d.um[0], d.vn[0], m_dev, cfg->rows, cfg->cols, h.pitch, G.south_open, d.T.ge_th,
                       cfg->g, &clk[cur].cmax_bits, b->stream));
    plan_kernel<<<1, 32, 0, b->stream>>>(G, F, clk, &b->d_scen[slot].ctl, cur);
    BCK(b, cudaGetLastError());
    ScenarioStatus s0;
    std::memset(&s0, 0, sizeof(s0));
    s0.running = 1;
    BCK(b, cudaMemcpyAsync(b->d_status + slot, &s0, sizeof(s0), cudaMemcpyHostToDevice, b->stream));
    h.active = true;
    int rc = upload_units(b);  // synchronises: the host-side sources above are safe to reuse
    if (rc) {  // the unit table is full: the scenario is not admitted and its memory goes back
        h.active = false;
        cudaFreeAsync(h.block, b->stream);
        h.block = nullptr;
        b->bytes_in_use -= (int64_t)h.bytes;
        h.bytes = 0;
        return rc;
    }
    *id = slot;
    return SW2D_OK;
}

int sw2d_batch_advance(sw2d_batch *b, int32_t launches, int32_t *running) {
    if (!b || launches < 0) return bfail(b, SW2D_ERR_INVALID_ARG, "bad arguments");
    BCK(b, cudaSetDevice(b->cfg.device));
    int left = launches;
    while (left > 0) {
        const int parity = (int)(b->launches % 3);
        if (left >= b->cfg.chunk) {
            if (!b->graph[parity]) {
                int rc = capture(b, parity);
                if (rc) return rc;
            }
            BCK(b, cudaGraphLaunch(b->graph[parity], b->stream));
            b->launches += b->cfg.chunk;
            left -= b->cfg.chunk;
        } else {
            BCK(b, launch_batch(b, parity));
            b->launches += 1;
            left -= 1;
        }
    }
    if (running) {
        BCK(b, cudaMemcpyAsync(b->h_status, b->d_status, b->scen.size() * sizeof(ScenarioStatus),
                               cudaMemcpyDeviceToHost, b->stream));
        BCK(b, cudaStreamSynchronize(b->stream));
        int n = 0;
        for (size_t s = 0; s < b->scen.size(); s++)
            if (b->scen[s].active && b->h_status[s].running) n++;
        *running = n;
    }
    return SW2D_OK;
}

int sw2d_batch_poll(sw2d_batch *b, int32_t *ids, int32_t *running, double *t, int64_t *steps, int32_t cap,
                    int32_t *n) {
    if (!b || !n) return bfail(b, SW2D_ERR_INVALID_ARG, "null argument");
    BCK(b, cudaMemcpyAsync(b->h_status, b->d_status, b->scen.size() * sizeof(ScenarioStatus), cudaMemcpyDeviceToHost,
                           b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    int k = 0;
    for (size_t s = 0; s < b->scen.size(); s++) {
        if (!b->scen[s].active) continue;
        if (k < cap) {
            if (ids) ids[k] = (int32_t)s;
            if (running) running[k] = b->h_status[s].running;
            if (t) t[k] = b->h_status[s].t;
            if (steps) steps[k] = b->h_status[s].steps;
        }
        k++;
        if (b->h_status[s].nonfinite) return bfail(b, SW2D_ERR_NONFINITE, "scenario produced a non-finite value");
    }
    *n = k;
    return SW2D_OK;
}

static int read_current_clock(sw2d_batch *b, const HostScenario &h) {
    const int cur = (int)(b->launches % 3);
    BCK(b, cudaMemcpyAsync(b->h_clk, h.dev.clk + cur, sizeof(Clock), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    return SW2D_OK;
}

int sw2d_batch_get_field(sw2d_batch *b, int32_t id, int32_t field, double *out) {
    if (!b || !out || id < 0 || id >= (int)b->scen.size() || !b->scen[id].active)
        return bfail(b, SW2D_ERR_INVALID_ARG, "bad scenario id");
    const HostScenario &h = b->scen[id];
    int rc = read_current_clock(b, h);
    if (rc) return rc;
    const int buf = b->h_clk->buf;
    const int rows = h.cfg.rows, cols = h.cfg.cols;
    int nr = rows, nc = cols;
    const float *src = nullptr, *add = nullptr;
    switch (field) {
    case SW2D_FIELD_DEPTH: src = h.dev.h[buf]; add = h.dev.hr[buf]; break;
    case SW2D_FIELD_UM: src = h.dev.um[buf]; nr = rows + 1; break;
    case SW2D_FIELD_VN: src = h.dev.vn[buf]; nc = cols + 1; break;
    case SW2D_FIELD_ELEVATION: src = h.dev.z; break;
    default: return bfail(b, SW2D_ERR_INVALID_ARG, "field not available for batched scenarios");
    }
    if (b->stage_elems < (size_t)nr * nc) return bfail(b, SW2D_ERR_STATE, "staging buffer too small");
    BCK(b, launch_unpack(src, add, nr, nc, h.pitch, b->d_stage, b->stream));
    BCK(b, cudaMemcpyAsync(out, b->d_stage, (size_t)nr * nc * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    BCK(b, cudaStreamSynchronize(b->stream));
    return SW2D_OK;
}


int sw2d_batch_get_budget(sw2d_batch *b, int32_t id, sw2d_budget *out) {
    if (!b || !out || id < 0 || id >= (int)b->scen.size() || !b->scen[id].active)
        return bfail(b, SW2D_ERR_INVALID_ARG, "bad scenario id");
    const HostScenario &h = b->scen[id];
    int rc = read_current_clock(b, h);
    if (rc) return rc;
    const Clock k = *b->h_clk;
    double vol = 0.0;
    rc = scenario_volume(b, h, k.buf, &vol);
    if (rc) return rc;
    double tot[B_N];
    for (int q = 0; q < B_N; q++) tot[q] = k.tot_s[q] + (k.step[q] - k.tot_c[q]);
    std::memset(out, 0, sizeof(*out));
    out->t = k.t;
    out->dt = k.dt;
    std::memcpy(&out->cmax, &k.cmax_bits, sizeof(double));
    out->volume = vol;
    out->volume0 = h.volume0;
    out->rain_in = tot[B_RAIN];
    out->source_in = tot[B_SRC];
    out->evap_out = tot[B_EV];
    out->outflow = tot[B_OUT];
    out->clamp_gain = tot[B_CLAMP];
    out->steps = k.steps;
    out->nonfinite = k.nonfinite ? 1 : 0;
    return SW2D_OK;
}

int sw2d_batch_remove(sw2d_batch *b, int32_t id) {
    if (!b || id < 0 || id >= (int)b->scen.size() || !b->scen[id].active)
        return bfail(b, SW2D_ERR_INVALID_ARG, "bad scenario id");
    HostScenario &h = b->scen[id];
    h.active = false;
    int rc = upload_units(b);  // the next launch no longer sees the scenario
    if (rc) return rc;
    BCK(b, cudaFreeAsync(h.block, b->stream));
    h.block = nullptr;
    b->bytes_in_use -= (int64_t)h.bytes;
    h.bytes = 0;
    return SW2D_OK;
}

int sw2d_batch_bytes_in_use(sw2d_batch *b, int64_t *bytes) {
    if (!b || !bytes) return SW2D_ERR_INVALID_ARG;
    *bytes = b->bytes_in_use;
    return SW2D_OK;
}

int sw2d_batch_get_stream(sw2d_batch *b, void **stream) {
    if (!b || !stream) return SW2D_ERR_INVALID_ARG;
    *stream = (void *)b->stream;
    return SW2D_OK;
}

int sw2d_batch_launch_count(sw2d_batch *b, int64_t *launches) {
    if (!b || !launches) return SW2D_ERR_INVALID_ARG;
    *launches = b->launches;
    return SW2D_OK;
}

const char *sw2d_batch_last_error(const sw2d_batch *b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"
