/*
 * sw2d.h -- C ABI of the GB300-native SW2D time-stepping core.
 *
 * This is the drop-in boundary for the solver loop of the reference
 * SW2D-GPU (SW2D-GPU_linux/src/SW2D-GPU.cu, "cu:<line>" below).  The
 * reference has no library interface: main() allocates 20 raw device arrays
 * (cu:1163-1190), uploads them (cu:1194-1213), launches nine kernels per
 * iteration (cu:1256-1336) and copies fields back for output
 * (cu:1376, 1426, 1442, 1458).  Each entry point below replaces one of those
 * steps; the comment on each names the reference code it stands in for.
 *
 * Conventions
 *   - Every call returns an int status (sw2d_status); nothing throws across
 *     the ABI.  sw2d_last_error() gives a message for the last failure.
 *   - Host arrays are row-major, north row first, float64:
 *       cells    rows x cols
 *       x-faces  (rows+1) x cols : um[i][j] is the face between cells
 *                (i-1,j) and (i,j); the reference's "X-DIRECTION" (cu:113)
 *       y-faces  rows x (cols+1) : vn[i][j] is the face between cells
 *                (i,j-1) and (i,j); the reference's "Y-DIRECTION" (cu:229)
 *     The device layout (pitch, precision) is private to the library.
 *   - The handle owns its device memory and one CUDA stream; the caller owns
 *     every host buffer.  A handle is not thread-safe.
 *   - A cell with elevation == nodata is inactive; all its faces are walls
 *     (cu:39-44, cu:117-118).
 */
#ifndef SW2D_H
#define SW2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SW2D_ABI_VERSION 1

typedef enum {
    SW2D_OK = 0,
    SW2D_ERR_INVALID_ARG = 1, /* bad size, null pointer, out-of-range value */
    SW2D_ERR_OOM = 2,         /* device allocation failed */
    SW2D_ERR_CUDA = 3,        /* any other CUDA runtime error */
    SW2D_ERR_NONFINITE = 4,   /* a NaN/Inf depth or discharge was produced */
    SW2D_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    SW2D_ERR_STATE = 6        /* call order: e.g. advance before set_static */
} sw2d_status;

enum { SW2D_PREC_F64 = 0, SW2D_PREC_F32 = 1 };
/* FIXED: the reference's rule, a constant half step dt (cu:790, cu:808),
 *        loop while t + dt <= t_end (cu:1256).
 * CFL:   extension; dt2 = min(2*dt, cfl*min(dx,dy)/cmax), clipped to t_end,
 *        where cmax = max over wet interior faces of |q/h_face| + sqrt(g*h_face)
 *        of the current state. */
enum { SW2D_DT_FIXED = 0, SW2D_DT_CFL = 1 };

/* Step kernels.  TILE: one CTA per 2-D tile staged in shared memory (the
 * FP64 path).  STREAM: one warp per 27-column strip marching down the rows
 * with a register pipeline (FP32 only).  AUTO: TILE for FP64, STREAM for FP32. */
enum { SW2D_KERNEL_AUTO = 0, SW2D_KERNEL_TILE = 1, SW2D_KERNEL_STREAM = 2 };

enum {
    SW2D_FIELD_DEPTH = 0,     /* h, rows x cols            (reference d_h)   */
    SW2D_FIELD_UM = 1,        /* x-face discharge, (rows+1) x cols (d_um)   */
    SW2D_FIELD_VN = 2,        /* y-face discharge, rows x (cols+1) (d_vn)   */
    SW2D_FIELD_UU = 3,        /* cell velocity along rows, rows x cols (d_uu, cu:473) */
    SW2D_FIELD_VV = 4,        /* cell velocity along cols, rows x cols (d_vv, cu:474) */
    SW2D_FIELD_ELEVATION = 5  /* z as stored on the device, rows x cols      */
};

enum {
    SW2D_RAIN_NONE = 0,
    SW2D_RAIN_COMPAT = 1, /* series in mm per interval, the reference's
                             interpolation formula (cu:547-554) */
    SW2D_RAIN_STEP = 2,   /* series in mm/h, constant over each interval, 0 after */
    SW2D_RAIN_LINEAR = 3, /* series in mm/h at knots k*dt, linear, 0 after */
    SW2D_RAIN_STORM = 4   /* moving Gaussian storm cell (sw2d_set_storm) */
};

typedef struct {
    int32_t rows, cols;
    double dx, dy;          /* cell size [m] (the reference has dx = dy = cellsize, cu:1236) */
    double nodata;          /* NODATA_value of the DEM (cu:827) */
    double g;               /* 9.80 in the reference (cu:809) */
    double th;              /* wet/dry threshold, 1.0e-4 m (cu:1130) */
    double manning;         /* scalar Manning n (cu:799) when no raster is given */
    double INT, INF, LWL;   /* runoff fractions of rain (cu:627-634) */
    double EV_WL_min;       /* depth above which LWL and evaporation apply */
    int32_t precision;      /* SW2D_PREC_F64 (exact scheme) or SW2D_PREC_F32 */
    int32_t dt_mode;        /* SW2D_DT_FIXED or SW2D_DT_CFL */
    double dt;              /* FIXED: the half step; CFL: the largest half step */
    double cfl;             /* Courant number for SW2D_DT_CFL (0.5) */
    int32_t south_open;     /* 1: free outfall through the south edge (extension) */
    int32_t device;         /* CUDA device ordinal */
    int32_t tile_h, tile_w; /* core tile of the shared-memory step kernel, 0 = default */
    int32_t kernel;         /* SW2D_KERNEL_*: which step kernel (AUTO picks per precision) */
    int32_t strip_h;        /* rows per warp of the FP32 streaming kernel, 0 = auto */
    int32_t variant;        /* streaming-kernel build (occupancy / unrolling), 0..6, 0 = default;
                               chosen by the autotuner among 0..5; 6 stages the rows in shared
                               memory by TMA (uniform forcing; the other forms run build 0);
                               every build gives the same state bits */
    int32_t steps_per_launch; /* iterations per kernel launch of the FP32 streaming kernel
                               (the reference launches nine kernels per iteration,
                               cu:1256-1336) under SW2D_DT_FIXED: K >= 2 runs K iterations per cooperative
                               launch, each warp starting its next iteration as soon as the
                               units around it have finished theirs (same state, bit for bit,
                               as one launch per iteration); 1 = one launch per iteration;
                               0 = the library's choice (48 where one wave of resident warps
                               holds the grid in strips of at most 32 rows -- grids up to
                               about 1600^2 -- and while neither a moving storm nor point
                               sources are set, else 1).  At most 1024; values >= 2 with
                               SW2D_DT_CFL or another kernel are SW2D_ERR_INVALID_ARG. */
} sw2d_config;

typedef struct {
    double t;          /* simulated time [s] */
    double dt;         /* half step of the last iteration [s] */
    double cmax;       /* wave-speed bound of the current state [m/s] */
    double volume;     /* water on active cells now [m^3], FP64 Kahan sum */
    double volume0;    /* at sw2d_set_state */
    double rain_in;    /* cumulative inflows/outflows [m^3], FP64 Kahan */
    double source_in;
    double evap_out;
    double outflow;    /* through the open south edge */
    double clamp_gain; /* water created by the depth clamp fmax(h,0) (cu:657) */
    int64_t steps;     /* iterations done since sw2d_set_state */
    int32_t nonfinite; /* 1 if a non-finite value was produced */
    int32_t reserved;
} sw2d_budget;

typedef struct sw2d_handle sw2d_handle;

/* Fills cfg with the reference's constants (g = 9.80, th = 1e-4, FP64,
 * fixed dt).  Replaces the constants of cu:808-809 and cu:1130. */
int sw2d_config_init(sw2d_config *cfg);

/* Device bytes a handle with this config allocates (admission control). */
int sw2d_device_bytes(const sw2d_config *cfg, int64_t *bytes);

/* Creates a handle and allocates all device memory.
 * Replaces the cudaMalloc block cu:1163-1190 and the launch setup cu:1222-1235. */
int sw2d_create(const sw2d_config *cfg, sw2d_handle **out);

/* Frees everything.  Replaces cu:1490-1521. */
int sw2d_destroy(sw2d_handle *h);

/* Uploads the DEM (rows x cols) and an optional per-cell Manning raster
 * (NULL = cfg.manning everywhere).  Derives the active mask.
 * Replaces the d_baseo upload (cu:1213) and init_inf (cu:29-49, cu:1238). */
int sw2d_set_static(sw2d_handle *h, const double *z, const double *manning);

/* Uploads the state at time t0: depth (rows x cols) and optional discharges
 * um ((rows+1) x cols) and vn (rows x (cols+1)); NULL = zero.  Inactive cells
 * get depth 0.  Resets budgets and the iteration count.
 * Replaces the state uploads cu:1194-1210 and initiald (cu:52-92, cu:1240). */
int sw2d_set_state(sw2d_handle *h, const double *depth, const double *um, const double *vn,
                   double t0);

/* Uniform rain series (SW2D_RAIN_COMPAT/STEP/LINEAR) or SW2D_RAIN_NONE.
 * Replaces the rain part of stream_flow (cu:547-554) and the d_rr uploads
 * (cu:1280, cu:1305). */
int sw2d_set_rain(sw2d_handle *h, int32_t kind, const double *series, int32_t n, double dt_series);

/* Moving Gaussian storm: rate = peak * exp(-r^2 / (2 sigma^2)) [mm/h] with
 * centre (x0 + vx t, y0 + vy t); x grows with the column, y with the row
 * (southwards), both from the north-west corner; zero for t >= t_stop.
 * Extension (the reference's rain is one scalar, cu:547). */
int sw2d_set_storm(sw2d_handle *h, double peak_mm_h, double x0, double y0, double vx,
                   double vy, double sigma, double t_stop);

/* Spatial rain distribution (extension for rainfall rasters; the reference
 * rains one interpolated value on every cell, cu:654): per-cell factors,
 * rows*cols values north row first, finite and >= 0, that multiply the rain
 * rate of whatever rain kind is set (series or storm), in both continuity
 * calls and in the rain budget.  NULL restores uniform rain.  Call after
 * sw2d_set_static, which clears the factors. */
int sw2d_set_rain_weights(sw2d_handle *h, const double *w);

/* Evaporation series in mm per interval, reference formula
 * (evaporation_load cu:589-601, d_Ev uploads cu:1284, cu:1309); applied
 * where the depth is above EV_WL_min (cu:627-634).  n = 0 disables it. */
int sw2d_set_evaporation(sw2d_handle *h, const double *series_mm, int32_t n, double dt_series);

/* The evaporation series of the reference's energy-balance method, in mm per
 * record interval, from n air temperatures [deg C] and global radiation
 * values [W/m^2]: replaces gpu_evaporation_calc (cu:557-587) and the copy of
 * its result to the host (cu:1242-1245).  A host computation (no handle, no
 * device): the same operations in the same order, without FMA contraction;
 * negative values become 0 (cu:583-585).  The result is what
 * sw2d_set_evaporation takes, with dt_series = dtime. */
int sw2d_evaporation_series(const double *temperature, const double *radiation, int32_t n, double albedo,
                            double dtime, double *evap_mm);

/* Point sources/sinks: cells[k] is the linear cell index i*cols+j of source
 * k; q is n_rec x n_src discharges [m^3/s] at interval dtoq, interpolated
 * with the reference's formula (stream_flow cu:532-546).  When two sources
 * share a cell the later one wins, as in the reference.  Replaces the d_ql
 * uploads (cu:1279, cu:1304).  n_src = 0 removes all sources. */
int sw2d_set_point_sources(sw2d_handle *h, const int32_t *cells, int32_t n_src, const double *q,
                           int32_t n_rec, double dtoq);

/* Runs iterations of the solver loop until max_steps iterations are done or
 * the end-time condition fails (FIXED: t + dt <= t_end as in cu:1256; CFL:
 * t < t_end, last step clipped to land on t_end).  *steps_done (nullable)
 * receives the count.  Replaces the while loop cu:1256-1336, which launches
 * nine kernels per iteration; here each iteration is one launch of the fused
 * step kernel, or cfg.steps_per_launch iterations share one cooperative
 * launch.  Returns SW2D_ERR_NONFINITE when a NaN/Inf was produced and
 * SW2D_ERR_TIMEOUT when a bounded wait inside such a launch gave up. */
int sw2d_advance(sw2d_handle *h, int64_t max_steps, double t_end, int64_t *steps_done);

/* Copies a field of the current state to host memory (size per field enum).
 * Replaces the D2H copies cu:1376, cu:1426, cu:1442, cu:1458; the velocity
 * fields are computed on demand (uu_vv, cu:459-484). */
int sw2d_get_field(sw2d_handle *h, int32_t field, double *out);

/* Time, step count and FP64 mass budget of the current state. */
int sw2d_get_budget(sw2d_handle *h, sw2d_budget *out);

/* Depth at n cells (linear indices i*cols + j; SW2D_ERR_INVALID_ARG if one
 * lies outside the grid).  Replaces the WaterLevel.txt probe loop
 * cu:1386-1410. */
int sw2d_probe(sw2d_handle *h, const int32_t *cells, int32_t n, double *out);

/* Checkpoint / restore (extension; the reference restarts only from a depth
 * raster, cu:1022-1033).  A checkpoint holds the state in the working
 * precision bit for bit (h, um, vn), the simulated time, the iteration count,
 * the CFL bound and the FP64 budgets, so that a handle restored from it
 * continues exactly as the one it was taken from.  It can be loaded into any
 * handle created with the same config (after sw2d_set_static). */
int sw2d_checkpoint_bytes(sw2d_handle *h, int64_t *bytes);
int sw2d_checkpoint_save(sw2d_handle *h, void *buf, int64_t bytes);
int sw2d_checkpoint_load(sw2d_handle *h, const void *buf, int64_t bytes);

/* Waits for all work of the handle.  The stream (a cudaStream_t) is
 * exposed so that callers can order their own work or time it. */
int sw2d_synchronize(sw2d_handle *h);
int sw2d_get_stream(sw2d_handle *h, void **stream);

/* Number of kernel launches of the time loop issued since sw2d_set_state:
 * one per iteration (including launches that found the run already finished
 * and did no work), or, with several iterations per launch, two per launch
 * (the plan kernel and the cooperative step kernel); plus, per advance, the
 * kernel that plans its first launch and, for the streaming kernel with one
 * launch per iteration, the one that folds the last launch's budgets. */
int sw2d_launch_count(sw2d_handle *h, int64_t *launches);

/* One line naming the step kernel build and the decomposition the handle
 * runs, e.g. "stream_step_kernel<2,10,2> forcing=uniform strip_h=52 units=3040
 * ctas=1520 steps_per_launch=1 strip_skew=20"
 * (written NUL-terminated, truncated to `n` bytes).  No reference
 * counterpart: the reference's launch shape is fixed at cu:1222-1235. */
int sw2d_describe(const sw2d_handle *h, char *buf, int32_t n);

const char *sw2d_last_error(const sw2d_handle *h);
const char *sw2d_status_string(int32_t status);

/* ---------------------------------------------------------------------------
 * Batched scenarios (extension; the reference runs one case at a time).
 *
 * A batch advances many FP32 scenarios of uneven size together: one
 * persistent launch per iteration whose warps pull (scenario, column tile,
 * row strip) units from a queue, each scenario with its own CFL time step,
 * clock, forcing and end time, all state resident on the device.  Scenarios
 * can be admitted (sw2d_batch_add) and retired (sw2d_batch_remove) between
 * advances; memory is allocated and released stream-ordered.  A scenario
 * advances bit for bit as it would alone in an FP32 handle.
 * ------------------------------------------------------------------------- */
typedef struct sw2d_batch sw2d_batch;

typedef struct {
    int32_t device;
    int32_t max_scenarios; /* size of the scenario table */
    int32_t max_units;     /* size of the work-unit table */
    int32_t strip_h;       /* rows per warp, 0 = by scenario size */
    int64_t max_bytes;     /* device budget for scenario data, 0 = none */
    int32_t chunk;         /* launches per CUDA-graph replay (multiple of 3) */
    int32_t variant;       /* build of the batched kernel, 0..2 (0 = default; the autotuner's choice) */
    int32_t reserved[2];
} sw2d_batch_config;

int sw2d_batch_config_init(sw2d_batch_config *cfg);
/* Device bytes one scenario of this shape takes in a batch (admission). */
int sw2d_batch_scenario_bytes(const sw2d_config *cfg, int32_t n_rain, int32_t with_raster, int64_t *bytes);
int sw2d_batch_create(const sw2d_batch_config *cfg, sw2d_batch **out);
int sw2d_batch_destroy(sw2d_batch *b);
/* Admits a scenario (cfg: FP32, CFL rule) starting at t = 0 with depth,
 * discharges 0, a uniform rain series and an end time; returns its id. */
int sw2d_batch_add(sw2d_batch *b, const sw2d_config *cfg, const double *z, const double *manning,
                   const double *depth, int32_t rain_kind, const double *rain, int32_t n_rain, double rain_dt,
                   double t_end, int32_t *id);
/* Enqueues `launches` iterations of every admitted scenario (finished ones
 * idle).  With running != NULL, waits and returns how many still run. */
int sw2d_batch_advance(sw2d_batch *b, int32_t launches, int32_t *running);
/* Status of the admitted scenarios (waits for queued work): up to cap
 * entries of id, running flag, simulated time and iterations; *n = count. */
int sw2d_batch_poll(sw2d_batch *b, int32_t *ids, int32_t *running, double *t, int64_t *steps, int32_t cap,
                    int32_t *n);
int sw2d_batch_get_field(sw2d_batch *b, int32_t id, int32_t field, double *out);
int sw2d_batch_get_budget(sw2d_batch *b, int32_t id, sw2d_budget *out);
int sw2d_batch_remove(sw2d_batch *b, int32_t id);
int sw2d_batch_bytes_in_use(sw2d_batch *b, int64_t *bytes);
int sw2d_batch_get_stream(sw2d_batch *b, void **stream);
int sw2d_batch_launch_count(sw2d_batch *b, int64_t *launches);
const char *sw2d_batch_last_error(const sw2d_batch *b);

/* ---------------------------------------------------------------------------
 * Continuous batching (extension): a serving loop over one batch, for a host
 * program that receives flood scenarios over time.
 *
 * Requests are submitted at any time.  Each sw2d_server_step admits the
 * waiting requests in submission order while the batch has a free scenario
 * slot (max_scenarios) and the request's device footprint
 * (sw2d_batch_scenario_bytes) fits the batch's max_bytes -- a request that
 * does not fit keeps its place and smaller ones behind it may pass it --,
 * advances every resident request by launches_per_step iterations, and
 * retires those whose end time is reached: their budgets (and, with
 * keep_depth, their depth raster) are copied to host memory and their device
 * memory is released at once.  A request advances bit for bit as it would
 * alone in an FP32 handle.  A request the batch refuses at admission (an
 * invalid argument or its memory) fails alone.  A server is not
 * thread-safe.
 * ------------------------------------------------------------------------- */
typedef struct sw2d_server sw2d_server;

typedef struct {
    sw2d_batch_config batch;   /* the batch: device, scenario slots, memory budget, kernel build */
    int32_t launches_per_step; /* iterations per sw2d_server_step, >= 1 (24) */
    int32_t keep_depth;        /* 1: keep each finished request's depth raster until released (1) */
    int32_t reserved[2];
} sw2d_server_config;

enum {
    SW2D_REQ_UNKNOWN = 0,   /* never submitted, or released */
    SW2D_REQ_PENDING = 1,   /* waiting for a slot and memory */
    SW2D_REQ_RUNNING = 2,   /* resident in the batch */
    SW2D_REQ_DONE = 3,      /* end time reached; results held until released */
    SW2D_REQ_FAILED = 4,    /* refused at admission (sw2d_server_request_error) */
    SW2D_REQ_CANCELLED = 5
};

int sw2d_server_config_init(sw2d_server_config *cfg);
int sw2d_server_create(const sw2d_server_config *cfg, sw2d_server **out);
int sw2d_server_destroy(sw2d_server *s);
/* Queues a request; the arguments are those of sw2d_batch_add.  The rasters
 * and the rain series are copied, so the caller's buffers may be reused on
 * return.  A request whose footprint exceeds the whole memory budget is
 * SW2D_ERR_INVALID_ARG.  *request: its id, 1, 2, ... */
int sw2d_server_submit(sw2d_server *s, const sw2d_config *cfg, const double *z, const double *manning,
                       const double *depth, int32_t rain_kind, const double *rain, int32_t n_rain, double rain_dt,
                       double t_end, int32_t *request);
/* One round -- admit, advance, retire -- and wait for it.  *pending and
 * *running (either may be NULL): the requests waiting and resident after it. */
int sw2d_server_step(sw2d_server *s, int32_t *pending, int32_t *running);
/* State (SW2D_REQ_*), simulated time and iterations of a request: as of the
 * last step while it runs, final once done.  t and steps may be NULL. */
int sw2d_server_poll(const sw2d_server *s, int32_t request, int32_t *state, double *t, int64_t *steps);
/* Results of a finished (SW2D_REQ_DONE) request: its FP64 budgets, and its
 * depth raster (rows x cols, kept with keep_depth). */
int sw2d_server_get_budget(const sw2d_server *s, int32_t request, sw2d_budget *out);
int sw2d_server_get_depth(const sw2d_server *s, int32_t request, double *out);
/* Withdraws a pending or running request (a running one leaves the batch
 * and its memory is released); SW2D_ERR_INVALID_ARG otherwise. */
int sw2d_server_cancel(sw2d_server *s, int32_t request);
/* Forgets a finished, failed or cancelled request and its results. */
int sw2d_server_release(sw2d_server *s, int32_t request);
/* Device bytes held by the resident requests. */
int sw2d_server_bytes_in_use(const sw2d_server *s, int64_t *bytes);
int sw2d_server_get_batch(sw2d_server *s, sw2d_batch **batch);  /* the underlying batch (stream, launch count) */
const char *sw2d_server_last_error(const sw2d_server *s);
/* Why a failed request was refused ("" for any other). */
const char *sw2d_server_request_error(const sw2d_server *s, int32_t request);

/* Largest grid sw2d_volume_noalloc accepts: 8192 x 8192 cells. */
#define SW2D_NOALLOC_MAX_CELLS (8192LL * 8192LL)

/* Volume of water [m^3] on the active cells of a depth field that the
 * caller already holds on the device, for callers that cannot allocate
 * device memory when they need the mass-balance check: a host model whose
 * own memory pool has reserved the whole GPU (a cudaMalloc there fails or
 * makes the pool give memory back), or one that must not call the allocator
 * inside its time loop (cudaMalloc and cudaFree can synchronise the device).
 * It allocates nothing: the partial sums live in a fixed 64 KiB array in the
 * library's device image (one per GPU that loads the library, held until
 * the process exits).  This entry point has no counterpart in the
 * reference, which keeps no mass budget.
 *
 *   depth      device pointer, rows x cols float64 with a row pitch of
 *              `pitch` elements (pitch >= cols)
 *   mask       device pointer with the same layout, 1 = active cell, or
 *              NULL when every cell counts
 *   cell_area  dx * dy [m^2]
 *   stream     cudaStream_t to run on (NULL = the legacy default stream)
 *
 * The call waits for its stream: the volume is on the host when it returns.
 * Returns SW2D_ERR_INVALID_ARG for null pointers, pitch < cols, a
 * non-positive cell area, or rows * cols > SW2D_NOALLOC_MAX_CELLS.  The sum
 * is deterministic (fixed chunks of 8192 cells, Kahan inside each chunk,
 * chunks added in order).  The first call in a CUDA context (one per device,
 * and again after the context is destroyed and made anew) looks up the
 * scratch array's device address; make that first call before any stream
 * capture.  Every call reuses the same scratch array: calls that overlap on
 * the GPU, from different streams or threads, race and must be serialised
 * by the caller. */
int sw2d_volume_noalloc(const double *depth, const uint8_t *mask, int32_t rows, int32_t cols, int32_t pitch,
                        double cell_area, void *stream, double *volume_out);

#ifdef __cplusplus
}
#endif

#endif /* SW2D_H */
