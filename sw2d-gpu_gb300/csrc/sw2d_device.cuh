// sw2d_device.cuh -- device-side types and the fused step kernel.
//
// One launch of step_kernel advances the whole domain by one iteration of
// the reference solver loop (SW2D-GPU_linux/src/SW2D-GPU.cu:1256-1336,
// "cu:<line>" below).  The reference runs that iteration as nine kernels
// with a host synchronisation after each and re-reads/re-writes 20 FP64
// arrays; here one CTA owns a TH x TW tile of cells, stages the tile plus a
// halo of 4 cells (north/west) and 3 cells (south/east) in shared memory
// and performs, entirely on chip:
//
//   stage 1  face depths hm/hn and face velocities uu1/vv1   (cu:363-453)
//   stage 2  new face discharges um/vn, momentum + dry bed   (cu:98-354)
//   stage 3  provisional depth h*, forcing at t              (cu:603-665)
//   stage 4  dry-cell outflow fix on each face (cu:695-725) and the final
//            depth, forcing at t+dt                           (cu:603-665)
//   stage 5  wave-speed bound of the new state (CFL rule, extension) and
//            the FP64 budget partials
//
// The transverse averages uua/vva (cu:490-523) are formed on the fly from
// uu1/vv1 in shared memory.  Only the state (h, um, vn) lives in HBM, in two
// ping-pong buffers; static fields (z, Manning n, active mask) are read-only.
//
// The dependency radius of one iteration is 3 cells (momentum needs h at
// i-2..i+1, the provisional depth needs the four new faces, the fix needs
// the provisional depth of both cells of a face).  One extra ring on the
// north/west sides gives the final depth of the neighbours of every owned
// face, so that the CFL bound of the NEW state is known when the launch
// ends and the next launch can pick its time step without a grid-wide
// synchronisation.
//
// The same template serves FP64 (compiled without FMA contraction, so that
// every operation rounds exactly as in the serial oracle and the reference
// built with --fmad=false) and FP32 (fast math).  Threshold tests are
// written as `x >= c` against host-computed constants so that the FP32 path
// decides wet/dry exactly as an FP64 comparison with th = 1e-4 would.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sw2d {

enum { B_RAIN = 0, B_SRC = 1, B_EV = 2, B_OUT = 3, B_CLAMP = 4, B_N = 5 };

// device-side status bits (sticky in the clock slots): more point sources in
// one warp window or tile than the kernel holds; a bounded wait of the
// pipelined launches gave up
enum { ST_TOO_MANY_LOCAL_SOURCES = 1, ST_PIPE_TIMEOUT = 2 };

constexpr int kMaxLocalSources = 64;
constexpr int kBuckets = 16;

// What one launch does, computed once per launch (never per thread: FP64
// arithmetic runs at a small fraction of the FP32 rate on this GPU).
template <class Real>
struct LaunchScalars {
    Real dt2;                  // 2 dt (cu:808)
    Real dt2dx, dt2dy;         // dt2/dx, dt2/dy as in cu:166, cu:283
    Real rr0, rr1, ev0, ev1;   // uniform rain / evaporation at t0 and t1 [m/s]
    Real sx0, sy0, sx1, sy1;   // storm centre at t0 and t1 [m]
};

struct Plan {
    int run, storm_on0, storm_on1, pad;
    double t0, t1, dt;         // t1 = t0 + dt (cu:1297)
    LaunchScalars<double> d;   // FP64 values
    LaunchScalars<float> f;    // the same, rounded once to FP32
};

// Per-iteration bookkeeping.  Three slots rotate: launch m reads slot m%3,
// accumulates into slot (m+1)%3, and its last CTA to finish finalises that
// slot (time, plan of launch m+1) and clears slot (m+2)%3 for launch m+1.
// No launch reads a slot that its own CTAs are still accumulating into, and
// no CTA ever waits for another.
struct __align__(16) Clock {
    double t;                      // time at the start of the next iteration
    double dt;                     // half step of the last iteration
    unsigned long long cmax_bits;  // CFL speed bound of this state (atomicMax on bits)
    long long steps;               // iterations since set_state
    int buf;                       // ping-pong buffer holding this state
    int ran;                       // the launch that wrote this slot advanced the state
    unsigned int nonfinite;        // a non-finite value was produced (sticky)
    unsigned int status;           // device-side error bits (sticky)
    double tot_s[B_N], tot_c[B_N]; // Kahan running totals of the budgets [m^3]
    double step[B_N];              // budget sums of the iteration that wrote this slot
    unsigned int done_blocks;      // CTAs of the writing launch that have finished
    unsigned int fold_pending;     // step and totals not yet folded (finalize_slot_deferred_warp)
    Plan plan;                     // what the launch reading this slot does
    // accumulators of the writing launch, spread over kBuckets addresses so
    // that thousands of CTAs do not serialise on one atomic location; summed
    // in bucket order by the last CTA
    double stepb[B_N][kBuckets];
    unsigned long long cmaxb[kBuckets];
};

struct Control {
    double t_end;
    long long step_limit;
};

template <class Real>
struct GridScalars {
    Real dx, dy, g, manning;
    Real rdx, rdy;             // 1/dx, 1/dy (used by the FP32 streaming kernel only)
    Real pct_hi, pct_lo;       // 1 - LWL and 1 - (INT + INF)   (cu:627-634)
    Real storm_amp, storm_2s2; // peak/3.6e6 [m/s] and 2 sigma^2 [m^2]
};

struct GridDesc {
    int rows, cols, pitch, tiles_w;
    int dt_mode, south_open, n_src, pad0;
    double dx, dy, g, th, cfl, dmin, dt_half;
    GridScalars<double> sd;    // FP64 values
    GridScalars<float> sf;     // the same, rounded once to FP32
};

template <class Real>
__device__ __forceinline__ const LaunchScalars<Real> &launch_scalars(const Plan &p);
template <>
__device__ __forceinline__ const LaunchScalars<double> &launch_scalars<double>(const Plan &p) { return p.d; }
template <>
__device__ __forceinline__ const LaunchScalars<float> &launch_scalars<float>(const Plan &p) { return p.f; }
template <class Real>
__device__ __forceinline__ const GridScalars<Real> &grid_scalars(const GridDesc &g);
template <>
__device__ __forceinline__ const GridScalars<double> &grid_scalars<double>(const GridDesc &g) { return g.sd; }
template <>
__device__ __forceinline__ const GridScalars<float> &grid_scalars<float>(const GridDesc &g) { return g.sf; }

struct ForcingDesc {
    int rain_kind, n_rain, n_ev, n_qrec;
    const double *rain;
    double rain_dt;
    double storm_peak, storm_x0, storm_y0, storm_vx, storm_vy, storm_sigma, storm_tstop;
    const double *ev;
    double ev_dt;
    const int *src_cell;
    const double *src_q;
    double dtoq;
};

template <class Real>
struct StateBufs {
    Real *h[2];
    Real *um[2];
    Real *vn[2];
    const Real *z;
    const Real *nman;  // per-cell Manning n or nullptr
    const uint8_t *mask;
    const Real *rainw;  // per-cell factors of the rain rate, or nullptr (uniform rain)
    const Real *dzx, *dzy;  // bed differences across x- / y-faces (streaming kernel only)
    Real *hr[2];            // depth remainders of the compensated FP32 state (streaming kernel only)
};

// wet/dry thresholds as `x >= c` constants (see file comment)
template <class Real>
struct Thr {
    Real gt_th;     // x > th      <=>  x >= gt_th
    Real ge_th;     // x >= th     <=>  x >= ge_th
    Real gt_evmin;  // x > EV_WL_min
};

enum { RAIN_NONE = 0, RAIN_COMPAT = 1, RAIN_STEP = 2, RAIN_LINEAR = 3, RAIN_STORM = 4 };

// ---------------------------------------------------------------------------
// time step decision, shared by host and device (one definition, so the host
// loop and every CTA decide identically)
// ---------------------------------------------------------------------------
__host__ __device__ inline bool decide_step(double t, double cmax, long long steps,
                                            const Control &ctl, const GridDesc &G,
                                            double *dt_half) {
    if (steps >= ctl.step_limit) return false;
    if (G.dt_mode == 0) {
        if (!(t + G.dt_half <= ctl.t_end)) return false;  // cu:1256
        *dt_half = G.dt_half;
        return true;
    }
    if (!(ctl.t_end - t > 1.0e-9)) return false;
    double dt2 = 2.0 * G.dt_half;
    if (cmax > 0.0) {
        double cand = G.cfl * G.dmin / cmax;
        if (cand < dt2) dt2 = cand;
    }
    if (t + dt2 > ctl.t_end) dt2 = ctl.t_end - t;
    *dt_half = 0.5 * dt2;
    return true;
}

// ---------------------------------------------------------------------------
// forcing (stream_flow cu:526-555, evaporation_load cu:589-601)
//
// The products and sums a compiler could fuse into one FMA are written with
// the _rn intrinsics, which it never fuses: the FP32 translation units
// compile with contraction on, and the plans they form (per launch, and in
// the pipelined launches' tables) must round exactly as the FP64 path's and
// the oracle's.
// ---------------------------------------------------------------------------
__device__ inline double compat_series(const double *v, int n, double dtv, double t) {
    if (n <= 0) return 0.0;
    if (t <= 1.00) return v[0] * t;
    int it = (int)(t / dtv);
    int a = it < n ? it : n - 1;
    int b = it + 1 < n ? it + 1 : n - 1;
    return v[a] + (v[b] - v[a]) / (dtv * __dsub_rn(t, __dmul_rn(dtv, (double)it)));
}

__device__ inline double rain_uniform(const ForcingDesc &F, double t) {
    switch (F.rain_kind) {
    case RAIN_COMPAT:
        return compat_series(F.rain, F.n_rain, F.rain_dt, t) / (F.rain_dt * 1000.0);
    case RAIN_STEP: {
        if (t < 0.0) return 0.0;
        long long k = (long long)floor(t / F.rain_dt);
        if (k >= F.n_rain) return 0.0;
        return F.rain[k] / 3.6e6;
    }
    case RAIN_LINEAR: {
        if (t < 0.0 || F.n_rain < 2) return 0.0;
        double s = t / F.rain_dt;
        long long k = (long long)floor(s);
        if (k >= F.n_rain - 1) return 0.0;
        double w = s - (double)k;
        return __dadd_rn(F.rain[k], __dmul_rn(w, F.rain[k + 1] - F.rain[k])) / 3.6e6;
    }
    default:
        return 0.0;
    }
}

__device__ inline double evap_rate(const ForcingDesc &F, double t) {
    if (F.n_ev <= 0) return 0.0;
    return compat_series(F.ev, F.n_ev, F.ev_dt, t) / (F.ev_dt * 1000.0);
}

__device__ inline double source_rate(const ForcingDesc &F, int n_src, int s, double t, double area) {
    double q;
    if (t <= 1.00) {
        q = F.src_q[s] * t;
    } else {
        int it = (int)(t / F.dtoq);
        int a = it < F.n_qrec ? it : F.n_qrec - 1;
        int b = it + 1 < F.n_qrec ? it + 1 : F.n_qrec - 1;
        double qa = F.src_q[(size_t)a * n_src + s];
        double qb = F.src_q[(size_t)b * n_src + s];
        q = qa + (qb - qa) / (F.dtoq * __dsub_rn(t, __dmul_rn(F.dtoq, (double)it)));
    }
    return q / area;
}

// One of the two evaluations a plan needs at time tl: the step over the cell
// size (dt2/dx for the x step, dt2/dy for the y step), the uniform rain and
// evaporation rates and the storm centre.  Inlined into both plan makers
// below, so that a plan is formed by the same operations either way.
struct PlanHalf {
    double q, rr, ev, sx, sy;
};

__device__ __forceinline__ PlanHalf plan_half(const GridDesc &G, const ForcingDesc &F, double dt2, double tl,
                                              bool second) {
    PlanHalf h;
    h.q = dt2 / (second ? G.dy : G.dx);
    h.rr = rain_uniform(F, tl);
    h.ev = evap_rate(F, tl);
    h.sx = __dadd_rn(F.storm_x0, __dmul_rn(F.storm_vx, tl));
    h.sy = __dadd_rn(F.storm_y0, __dmul_rn(F.storm_vy, tl));
    return h;
}

__device__ __forceinline__ void plan_round(Plan &p) {
    const LaunchScalars<double> &d = p.d;
    LaunchScalars<float> &f = p.f;
    f.dt2 = (float)d.dt2;
    f.dt2dx = (float)d.dt2dx;
    f.dt2dy = (float)d.dt2dy;
    f.rr0 = (float)d.rr0;
    f.rr1 = (float)d.rr1;
    f.ev0 = (float)d.ev0;
    f.ev1 = (float)d.ev1;
    f.sx0 = (float)d.sx0;
    f.sy0 = (float)d.sy0;
    f.sx1 = (float)d.sx1;
    f.sy1 = (float)d.sy1;
}

__device__ __forceinline__ void plan_clear(Plan &p, double t) {
    p.run = 0;
    p.storm_on0 = p.storm_on1 = 0;
    p.pad = 0;
    p.t0 = t;
    p.t1 = t;
    p.dt = 0.0;
    LaunchScalars<double> &d = p.d;
    d.dt2 = d.dt2dx = d.dt2dy = 0.0;
    d.rr0 = d.rr1 = d.ev0 = d.ev1 = 0.0;
    d.sx0 = d.sy0 = d.sx1 = d.sy1 = 0.0;
}

// The plan of the launch that reads clock slot c under control ctl.  Called
// by all 32 lanes of one converged warp; every lane returns the same plan.
// FP64 arithmetic on this GPU has long latencies (a division takes several
// hundred cycles) and the plan lies on the critical path between two
// launches, so the pairs of independent evaluations -- the forcing at t0 and
// at t1, dt2/dx and dt2/dy -- run as one instruction stream on lanes 0 and 1
// instead of one after the other.  Each value is computed by the same
// operations as a serial evaluation would use (make_plan_serial).
__device__ inline Plan make_plan_warp(const int lane, double t, unsigned long long cmax_bits, long long steps,
                                      const Control &ctl, const GridDesc &G, const ForcingDesc &F) {
    Plan p;
    plan_clear(p, t);
    LaunchScalars<double> &d = p.d;
    double dt = 0.0;
    if (decide_step(t, __longlong_as_double((long long)cmax_bits), steps, ctl, G, &dt)) {  // warp-uniform
        p.run = 1;
        p.dt = dt;
        p.t1 = t + dt;
        d.dt2 = 2.00 * dt;
        const bool second = (lane & 1) != 0;  // lane 1: t1 and the y step; lane 0: t0 and the x step
        const PlanHalf h = plan_half(G, F, d.dt2, second ? p.t1 : p.t0, second);
        d.dt2dx = __shfl_sync(0xffffffffu, h.q, 0);
        d.dt2dy = __shfl_sync(0xffffffffu, h.q, 1);
        d.rr0 = __shfl_sync(0xffffffffu, h.rr, 0);
        d.rr1 = __shfl_sync(0xffffffffu, h.rr, 1);
        d.ev0 = __shfl_sync(0xffffffffu, h.ev, 0);
        d.ev1 = __shfl_sync(0xffffffffu, h.ev, 1);
        if (F.rain_kind == RAIN_STORM) {
            p.storm_on0 = p.t0 < F.storm_tstop;
            p.storm_on1 = p.t1 < F.storm_tstop;
            d.sx0 = __shfl_sync(0xffffffffu, h.sx, 0);
            d.sy0 = __shfl_sync(0xffffffffu, h.sy, 0);
            d.sx1 = __shfl_sync(0xffffffffu, h.sx, 1);
            d.sy1 = __shfl_sync(0xffffffffu, h.sy, 1);
        }
    }
    plan_round(p);
    return p;
}

// The same plan from one thread (the pipelined launches' plan tables).
__device__ inline Plan make_plan_serial(double t, unsigned long long cmax_bits, long long steps, const Control &ctl,
                                        const GridDesc &G, const ForcingDesc &F) {
    Plan p;
    plan_clear(p, t);
    LaunchScalars<double> &d = p.d;
    double dt = 0.0;
    if (decide_step(t, __longlong_as_double((long long)cmax_bits), steps, ctl, G, &dt)) {
        p.run = 1;
        p.dt = dt;
        p.t1 = t + dt;
        d.dt2 = 2.00 * dt;
        const PlanHalf h0 = plan_half(G, F, d.dt2, p.t0, false);
        const PlanHalf h1 = plan_half(G, F, d.dt2, p.t1, true);
        d.dt2dx = h0.q;
        d.dt2dy = h1.q;
        d.rr0 = h0.rr;
        d.rr1 = h1.rr;
        d.ev0 = h0.ev;
        d.ev1 = h1.ev;
        if (F.rain_kind == RAIN_STORM) {
            p.storm_on0 = p.t0 < F.storm_tstop;
            p.storm_on1 = p.t1 < F.storm_tstop;
            d.sx0 = h0.sx;
            d.sy0 = h0.sy;
            d.sx1 = h1.sx;
            d.sy1 = h1.sy;
        }
    }
    plan_round(p);
    return p;
}

// ---------------------------------------------------------------------------
// clock-slot bookkeeping shared by the step kernels
// ---------------------------------------------------------------------------
__device__ inline void clear_slot_accumulators(Clock &c) {
    c.cmax_bits = 0ull;
    c.nonfinite = 0u;
    c.status = 0u;
    c.done_blocks = 0u;
    for (int k = 0; k < B_N; k++) {
        c.step[k] = 0.0;
        for (int b = 0; b < kBuckets; b++) c.stepb[k][b] = 0.0;
    }
    for (int b = 0; b < kBuckets; b++) c.cmaxb[b] = 0ull;
}

// The same, by the lanes of one warp: lane b clears bucket b.
__device__ inline void clear_slot_accumulators_warp(const int lane, Clock &c) {
    if (lane < kBuckets) {
        c.cmaxb[lane] = 0ull;
        for (int k = 0; k < B_N; k++) c.stepb[k][lane] = 0.0;
    }
    if (lane == 0) {
        c.cmax_bits = 0ull;
        c.nonfinite = 0u;
        c.status = 0u;
        c.done_blocks = 0u;
        for (int k = 0; k < B_N; k++) c.step[k] = 0.0;
    }
}

__device__ inline void fold_totals(const Clock &ci, Clock &co) {
    for (int k = 0; k < B_N; k++) {  // Kahan: running total += previous iteration's sum
        double s = ci.tot_s[k], c = ci.tot_c[k];
        double y = ci.step[k] - c;
        double tt = s + y;
        co.tot_c[k] = (tt - s) - y;
        co.tot_s[k] = tt;
    }
}

// A launch whose plan says "do not run": one thread carries the state's
// clock to the next slot unchanged.
__device__ inline void carry_slot(const Clock &ci, Clock &co, Clock &cn) {
    fold_totals(ci, co);
    co.t = ci.t;
    co.dt = ci.dt;
    co.steps = ci.steps;
    co.buf = ci.buf;
    co.ran = 0;
    co.cmax_bits = ci.cmax_bits;
    co.nonfinite = ci.nonfinite;
    co.status = ci.status;
    co.plan = ci.plan;
    for (int k = 0; k < B_N; k++) co.step[k] = 0.0;
    clear_slot_accumulators(cn);
}

// One CTA's contribution (one thread calls it): budget sums [m^3 already
// scaled], CFL bound, non-finite flag.
__device__ inline void accumulate_slot(Clock &co, int bucket, const double v[B_N], double cmax, bool bad) {
    for (int k = 0; k < B_N; k++)
        if (v[k] != 0.0) atomicAdd(&co.stepb[k][bucket], v[k]);
    if (cmax > 0.0) atomicMax(&co.cmaxb[bucket], (unsigned long long)__double_as_longlong(cmax));
    if (bad) atomicOr(&co.nonfinite, 1u);
}

// Finalises slot `co` once every contribution of the launch is in: sums the
// buckets, folds the budgets, advances time, plans the next launch, and
// clears slot `cn` for the launch after.  Called by all 32 lanes of one
// converged warp: lane b reads bucket b, and a shuffle tree (the same in
// every lane) takes their maximum and sums; lane 0 writes the slot.  `pl` is
// the plan of the launch's last iteration and `iters` the number of
// iterations the launch ran (more than one for the pipelined launches).
__device__ inline void finalize_slot_warp(const int lane, const Clock &ci, Clock &co, Clock &cn, const Plan &pl,
                                          const Control &ctl, const GridDesc &G, const ForcingDesc &F,
                                          const int iters = 1) {
    volatile Clock *cov = &co;
    unsigned long long cm = 0ull;
    double sum[B_N];
    for (int k = 0; k < B_N; k++) sum[k] = 0.0;
    if (lane < kBuckets) {
        cm = cov->cmaxb[lane];
        for (int k = 0; k < B_N; k++) sum[k] = cov->stepb[k][lane];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long c2 = __shfl_xor_sync(0xffffffffu, cm, o);
        cm = c2 > cm ? c2 : cm;
#pragma unroll
        for (int k = 0; k < B_N; k++) sum[k] += __shfl_xor_sync(0xffffffffu, sum[k], o);
    }
    const double t_new = (pl.t0 + pl.dt) + pl.dt;  // cu:1297, cu:1335
    const long long steps_new = ci.steps + iters;
    const Plan np = make_plan_warp(lane, t_new, cm, steps_new, ctl, G, F);
    if (lane == 0) {
        for (int k = 0; k < B_N; k++) co.step[k] = sum[k];
        fold_totals(ci, co);
        co.cmax_bits = cm;
        co.t = t_new;
        co.dt = pl.dt;
        co.steps = steps_new;
        co.buf = ci.buf ^ (iters & 1);
        co.ran = 1;
        co.nonfinite = cov->nonfinite | ci.nonfinite;
        co.status = cov->status | ci.status;
        co.plan = np;
    }
    clear_slot_accumulators_warp(lane, cn);
}

// Called by all 32 lanes of one warp of every CTA after lane 0's
// accumulate_slot; the last CTA of the launch finalises the slot.  No CTA
// waits.
__device__ inline void finish_cta_warp(const int lane, const Clock &ci, Clock &co, Clock &cn, const Plan &pl,
                                       const Control &ctl, const GridDesc &G, const ForcingDesc &F,
                                       const int iters = 1) {
    unsigned int ticket = 0u;
    if (lane == 0) {
        __threadfence();
        ticket = atomicAdd(&co.done_blocks, 1u);
    }
    ticket = __shfl_sync(0xffffffffu, ticket, 0);
    if (ticket != gridDim.x * gridDim.y - 1) return;
    __threadfence();
    finalize_slot_warp(lane, ci, co, cn, pl, ctl, G, F, iters);
}

// ---- the same bookkeeping with the budget fold off the critical path ----
//
// The last CTA of a launch lies on the critical path between two launches;
// of the slot it finalises, the next launch needs only the time, the step
// count, the buffer and the plan (from the CFL bound).  The budget sums --
// five FP64 shuffle trees and the Kahan fold, several microseconds of
// FP64 latency on one warp -- are left in the slot's buckets and folded by
// the FIRST CTA to finish the next launch (fold_slot_warp), tens of
// microseconds before that launch ends, or by fold_kernel after the host's
// last launch.  A fold reads the slot's buckets and the previous slot's
// step and totals, all final by then, and writes only the slot's own step
// and totals; the slot's fold_pending flag makes it happen once (a slot
// set by the host -- a new state, a restored checkpoint -- has nothing to
// fold), and the accumulators a launch clears for the launch after leave
// step and totals alone.

// Folds slot c, written by the launch that read slot prev: c.step = its
// bucket sums (the shuffle tree of finalize_slot_warp), c.tot = prev.tot +
// prev.step (Kahan).  All 32 lanes of one converged warp.
__device__ inline void fold_slot_warp(const int lane, const Clock &prev, Clock &c) {
    volatile Clock *cv = &c;
    if (cv->fold_pending == 0u) return;  // the same value in every lane
    double sum[B_N];
    for (int k = 0; k < B_N; k++) sum[k] = lane < kBuckets ? cv->stepb[k][lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < B_N; k++) sum[k] += __shfl_xor_sync(0xffffffffu, sum[k], o);
    }
    if (lane == 0) {
        for (int k = 0; k < B_N; k++) c.step[k] = sum[k];
        fold_totals(prev, c);
        c.fold_pending = 0u;
    }
}

// clear_slot_accumulators_warp without the step sums (see above).
__device__ inline void clear_slot_buckets_warp(const int lane, Clock &c) {
    if (lane < kBuckets) {
        c.cmaxb[lane] = 0ull;
        for (int k = 0; k < B_N; k++) c.stepb[k][lane] = 0.0;
    }
    if (lane == 0) {
        c.cmax_bits = 0ull;
        c.nonfinite = 0u;
        c.status = 0u;
        c.done_blocks = 0u;
    }
}

// finalize_slot_warp for one iteration without the budgets: the CFL bound
// (an integer maximum of the buckets' bits), time, plan, flags.
__device__ inline void finalize_slot_deferred_warp(const int lane, const Clock &ci, Clock &co, Clock &cn,
                                                   const Plan &pl, const Control &ctl, const GridDesc &G,
                                                   const ForcingDesc &F) {
    volatile Clock *cov = &co;
    unsigned long long cm = lane < kBuckets ? cov->cmaxb[lane] : 0ull;
    unsigned int nf = lane == 16 ? cov->nonfinite : 0u;
    unsigned int st = lane == 17 ? cov->status : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long c2 = __shfl_xor_sync(0xffffffffu, cm, o);
        cm = c2 > cm ? c2 : cm;
    }
    nf = __shfl_sync(0xffffffffu, nf, 16);
    st = __shfl_sync(0xffffffffu, st, 17);
    const double t_new = (pl.t0 + pl.dt) + pl.dt;  // cu:1297, cu:1335
    const long long steps_new = ci.steps + 1;
    const Plan np = make_plan_warp(lane, t_new, cm, steps_new, ctl, G, F);
    if (lane == 0) {
        co.cmax_bits = cm;
        co.t = t_new;
        co.dt = pl.dt;
        co.steps = steps_new;
        co.buf = 1 - ci.buf;
        co.ran = 1;
        co.nonfinite = nf | ci.nonfinite;
        co.status = st | ci.status;
        co.plan = np;
        co.fold_pending = 1u;
    }
    clear_slot_buckets_warp(lane, cn);
}

// finish_cta_warp with the deferred fold: the first CTA to finish folds the
// slot this launch read (written by the previous launch), the last
// finalises the slot this launch wrote.  clk, and the three slot indices as
// in the step kernels.
__device__ inline void finish_cta_deferred_warp(const int lane, Clock *clk, const int slot, const int slot_out,
                                                const int slot_nx, const Plan &pl, const Control &ctl,
                                                const GridDesc &G, const ForcingDesc &F) {
    unsigned int ticket = 0u;
    if (lane == 0) {
        __threadfence();
        ticket = atomicAdd(&clk[slot_out].done_blocks, 1u);
    }
    ticket = __shfl_sync(0xffffffffu, ticket, 0);
    const unsigned int last = gridDim.x * gridDim.y - 1;
    if (ticket == 0u) fold_slot_warp(lane, clk[slot_nx], clk[slot]);
    if (ticket != last) return;
    __threadfence();
    finalize_slot_deferred_warp(lane, clk[slot], clk[slot_out], clk[slot_nx], pl, ctl, G, F);
}

// A launch whose plan says "do not run", with the deferred fold: one warp
// folds the slot it read, then carries it (carry_slot).
__device__ inline void carry_slot_deferred_warp(const int lane, Clock *clk, const int slot, const int slot_out,
                                                const int slot_nx) {
    fold_slot_warp(lane, clk[slot_nx], clk[slot]);
    __syncwarp();
    if (lane == 0) carry_slot(clk[slot], clk[slot_out], clk[slot_nx]);
}

// Folds slot `slot` (see above) after the last launch the host issued.
static __global__ void fold_kernel(Clock *__restrict__ clk, const int slot, const int prev) {
    fold_slot_warp((int)threadIdx.x, clk[prev], clk[slot]);
}

// ---------------------------------------------------------------------------
// deterministic FP64 log / exp / power.  Same algorithm, operation order and
// tables as the oracle's, compiled without FMA contraction, so the FP64 path
// and the oracle agree to the bit where the reference uses pow (cu:195,
// cu:312).  The update uses the table-driven forms: log with 1/c and ln c for
// c = 1 + k/128 (k = the top 7 bits of the mantissa) and the series of
// ln(1+r) to r^8/8; exp with a reduction by ln2/64, the series of e^r to
// r^6/6! and 2^(j/64).  The tables are built by det_tables_kernel from the
// series forms (log: atanh series on [1/sqrt2, sqrt2) to s^21/21; exp:
// Cody-Waite by ln2, Taylor to r^13/13!) in each translation unit that uses
// them (init_det_tables).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double det_log_series(double x) {
    const long long b = __double_as_longlong(x);
    int e = (int)((b >> 52) & 0x7ff) - 1023;
    double m = __longlong_as_double((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double p = 1.0 / 21.0;
    p = p * s2 + 1.0 / 19.0;
    p = p * s2 + 1.0 / 17.0;
    p = p * s2 + 1.0 / 15.0;
    p = p * s2 + 1.0 / 13.0;
    p = p * s2 + 1.0 / 11.0;
    p = p * s2 + 1.0 / 9.0;
    p = p * s2 + 1.0 / 7.0;
    p = p * s2 + 1.0 / 5.0;
    p = p * s2 + 1.0 / 3.0;
    p = p * s2 + 1.0;
    const double lm = 2.0 * s * p;
    const double ef = (double)e;
    return ef * 0x1.62e42p-1 + (ef * 0x1.fdf473de6af28p-22 + lm);
}

__device__ __forceinline__ double det_exp_series(double y) {
    const double kf = floor(y * 0x1.71547652b82fep+0 + 0.5);
    const double r = (y - kf * 0x1.62e42p-1) - kf * 0x1.fdf473de6af28p-22;
    double p = 1.0 / 6227020800.0;
    p = p * r + 1.0 / 479001600.0;
    p = p * r + 1.0 / 39916800.0;
    p = p * r + 1.0 / 3628800.0;
    p = p * r + 1.0 / 362880.0;
    p = p * r + 1.0 / 40320.0;
    p = p * r + 1.0 / 5040.0;
    p = p * r + 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    const int k = (int)kf;
    return p * __longlong_as_double((long long)(k + 1023) << 52);
}

// [0,128): 1/c_k, [128,256): ln c_k, [256,320): 2^(j/64); one copy per
// translation unit, filled by det_tables_kernel before the first use
static __device__ double g_det_tab[320];

static __global__ void det_tables_kernel() {
    const int t = threadIdx.x;
    if (t < 128) {
        const double c = 1.0 + (double)t * 0.0078125;
        g_det_tab[t] = 1.0 / c;
        g_det_tab[128 + t] = det_log_series(c);
    }
    if (t < 64)
        g_det_tab[256 + t] = det_exp_series((double)t * (0x1.62e42p-1 / 64.0) + (double)t * (0x1.fdf473de6af28p-22 / 64.0));
}

__device__ __forceinline__ double det_log(double x) {
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    const int k = (int)((b >> 45) & 127);
    const double m = __longlong_as_double((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
    const double c = 1.0 + (double)k * 0.0078125;
    const double r = (m - c) * __ldg(&g_det_tab[k]);
    double p = -1.0 / 8.0;
    p = p * r + 1.0 / 7.0;
    p = p * r - 1.0 / 6.0;
    p = p * r + 1.0 / 5.0;
    p = p * r - 1.0 / 4.0;
    p = p * r + 1.0 / 3.0;
    p = p * r - 0.5;
    p = p * r + 1.0;
    const double lr = p * r;
    const double ef = (double)e;
    return ef * 0x1.62e42p-1 + (ef * 0x1.fdf473de6af28p-22 + (__ldg(&g_det_tab[128 + k]) + lr));
}

__device__ __forceinline__ double det_exp(double y) {
    if (y < -700.0) return 0.0;
    if (y > 700.0) return __longlong_as_double(0x7ff0000000000000LL);
    const double nf = floor(y * (64.0 * 0x1.71547652b82fep+0) + 0.5);
    const double r = (y - nf * (0x1.62e42p-1 / 64.0)) - nf * (0x1.fdf473de6af28p-22 / 64.0);
    double p = 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    const int n = (int)nf;
    const int j = n & 63, q = (n - j) / 64;  // n = 64 q + j, 0 <= j < 64
    return (p * __ldg(&g_det_tab[256 + j])) * __longlong_as_double((long long)(q + 1023) << 52);
}

// ---------------------------------------------------------------------------
// precision traits
// ---------------------------------------------------------------------------
template <class Real>
struct RT;

template <>
struct RT<double> {
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
    static __device__ __forceinline__ double pow_(double x) { return det_exp(1.3333330 * det_log(x)); }  // cu:195
    static __device__ __forceinline__ double exp_(double x) { return det_exp(x); }
    static __device__ __forceinline__ bool finite_(double x) { return isfinite(x); }
};

template <>
struct RT<float> {
    static __device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float pow_(float x) { return __powf(x, 1.3333330f); }
    static __device__ __forceinline__ float exp_(float x) { return __expf(x); }
    static __device__ __forceinline__ bool finite_(float x) { return isfinite(x); }
};

// Dry-bed rules (cu:130-159 / cu:247-276).  `a` is the low-index cell of the
// face (north / west), `b` the high-index cell.  Returns true and sets q
// when a rule applies; false means "use the momentum equation".
template <class Real>
__device__ __forceinline__ bool dry_bed(const Thr<Real> &T, Real g, Real ha, Real za, Real hb,
                                        Real zb, Real &q) {
    if (hb + zb < za) {  // cu:130
        q = (ha >= T.gt_th) ? Real(0.5440) * ha * RT<Real>::sqrt_(g * ha) : Real(0);
        return true;
    }
    if (ha + za < zb) {  // cu:138
        q = (hb >= T.gt_th) ? Real(-0.544) * hb * RT<Real>::sqrt_(g * hb) : Real(0);
        return true;
    }
    // cu:149: (hb - th) * (ha - th) < 0, i.e. exactly one side strictly wet;
    // written with comparisons that are false for NaN, as the product is
    const bool b_wet = hb >= T.gt_th, a_wet = ha >= T.gt_th;
    const bool b_dry = hb < T.ge_th, a_dry = ha < T.ge_th;
    if ((b_wet && a_dry) || (b_dry && a_wet)) {
        if ((hb > Real(0)) || (ha > Real(0))) {
            // -sgn(hb - ha) * 0.350 with sgn from the wet side (cu:151-154)
            const Real s = b_wet ? Real(-0.350) : Real(0.350);
            const Real ea = ha + za, eb = hb + zb;
            const Real hh3 = fmax(eb, ea) - fmax(zb, za);
            q = s * hh3 * RT<Real>::sqrt_(Real(2.00) * g * hh3);
        } else {
            q = Real(0);
        }
        return true;
    }
    return false;
}

// upwinded flux through one side of a control volume (pattern of cu:174)
template <class Real>
__device__ __forceinline__ Real upwind(Real vel, Real q_other, Real q_self) {
    return vel * (q_other + q_self) * Real(0.50) + fabs(vel) * (q_self - q_other) * Real(0.50);
}
template <class Real>
__device__ __forceinline__ Real upwind_r(Real vel, Real q_other, Real q_self) {
    // same with the operand order of the "left"/"down" sides (cu:175, cu:188)
    return vel * (q_self + q_other) * Real(0.50) + fabs(vel) * (q_other - q_self) * Real(0.50);
}

// ---------------------------------------------------------------------------
// the fused step kernel
// ---------------------------------------------------------------------------
template <class Real, int TH, int TW>
constexpr size_t step_smem_bytes() {
    return (size_t)(TH + 7) * (TW + 7) * (10 * sizeof(Real) + 1) + 64;
}

template <class Real, int TH, int TW, int NT>
__global__ void __launch_bounds__(NT)
    step_kernel(const GridDesc G, const ForcingDesc F, const StateBufs<Real> S, const Thr<Real> T,
                Clock *__restrict__ clk, const Control *__restrict__ ctl, const int slot) {
    constexpr int HN = 4;                       // halo north/west (3 + CFL ring)
    constexpr int RH = TH + 7, RW = TW + 7, RN = RH * RW;
    constexpr int NW = NT / 32;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real *s_h = reinterpret_cast<Real *>(smem_raw);
    Real *s_z = s_h + RN;
    Real *s_umo = s_z + RN;  // old um, later the corrected new um
    Real *s_vno = s_umo + RN;
    Real *s_uu1 = s_vno + RN;
    Real *s_vv1 = s_uu1 + RN;
    Real *s_rum = s_vv1 + RN;  // new um before the dry-cell fix
    Real *s_rvn = s_rum + RN;
    Real *s_hs = s_rvn + RN;   // provisional depth
    Real *s_n = s_hs + RN;     // Manning n per cell (only if G has a raster)
    uint8_t *s_m = reinterpret_cast<uint8_t *>(s_n + RN);

    __shared__ Real s_red[NW][B_N + 1];
    __shared__ int s_nloc;
    __shared__ int s_srcp[kMaxLocalSources];
    __shared__ Real s_srcq0[kMaxLocalSources], s_srcq1[kMaxLocalSources];
    __shared__ int s_wcnt[NW];

    const int tid = threadIdx.x;
    const int slot_out = slot == 2 ? 0 : slot + 1;
    const int slot_nx = slot == 0 ? 2 : slot - 1;
    const Clock &ci = clk[slot];
    const Plan pl = ci.plan;

    if (!pl.run) {  // nothing to do: carry the state's clock forward
        if (blockIdx.x == 0 && tid == 0) carry_slot(ci, clk[slot_out], clk[slot_nx]);
        return;
    }

    const int rows = G.rows, cols = G.cols, pitch = G.pitch;
    const int ti = blockIdx.x / G.tiles_w, tj = blockIdx.x - ti * G.tiles_w;
    const int I0 = ti * TH - HN, J0 = tj * TW - HN;  // global index of smem (0,0)
    const int buf = ci.buf;
    const Real *__restrict__ Hin = S.h[buf];
    const Real *__restrict__ Uin = S.um[buf];
    const Real *__restrict__ Vin = S.vn[buf];
    Real *__restrict__ Hout = S.h[1 - buf];
    Real *__restrict__ Uout = S.um[1 - buf];
    Real *__restrict__ Vout = S.vn[1 - buf];
    const bool has_n = S.nman != nullptr;

    const LaunchScalars<Real> LS = launch_scalars<Real>(pl);
    const GridScalars<Real> &GS = grid_scalars<Real>(G);
    const Real dt2 = LS.dt2;
    const Real dx = GS.dx, dy = GS.dy, g = GS.g;
    const Real dt2dx = LS.dt2dx, dt2dy = LS.dt2dy;
    const Real manning = GS.manning;

    // ---- stage 0: stage the tile + halo in shared memory --------------------
    for (int idx = tid; idx < RN; idx += NT) {
        const int r = idx / RW, c = idx - (idx / RW) * RW;
        const int gi = I0 + r, gj = J0 + c;
        const bool in_r = (unsigned)gi < (unsigned)rows, in_c = (unsigned)gj < (unsigned)cols;
        const size_t gp = (size_t)gi * pitch + gj;
        Real hv = 0, zv = 0, nv = 0;
        uint8_t mv = 0;
        if (in_r && in_c) {
            hv = Hin[gp];
            zv = S.z[gp];
            mv = S.mask[gp];
            if (has_n) nv = S.nman[gp];
        }
        s_h[idx] = hv;
        s_z[idx] = zv;
        s_m[idx] = mv;
        if (has_n) s_n[idx] = nv;
        s_umo[idx] = ((unsigned)gi <= (unsigned)rows && in_c) ? Uin[gp] : Real(0);
        s_vno[idx] = (in_r && (unsigned)gj <= (unsigned)cols) ? Vin[gp] : Real(0);
    }
    if (tid == 0) s_nloc = 0;
    // point sources inside this tile's provisional-depth region, kept in
    // list order so that a later source on the same cell wins (cu:545)
    if (G.n_src > 0) {
        __syncthreads();
        const double area = G.dx * G.dy;
        for (int base = 0; base < G.n_src; base += NT) {
            const int s = base + tid;
            bool in = false;
            int p = 0;
            if (s < G.n_src) {
                const int cell = F.src_cell[s];
                const int gi = cell / cols, gj = cell - (cell / cols) * cols;
                const int r = gi - I0, c = gj - J0;
                in = (r >= 2 && r < TH + 5 && c >= 2 && c < TW + 5);
                p = r * RW + c;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            const int lane = tid & 31, wid = tid >> 5;
            if (lane == 0) s_wcnt[wid] = __popc(bal);
            __syncthreads();
            if (in) {
                int off = s_nloc;
                for (int w = 0; w < wid; w++) off += s_wcnt[w];
                off += __popc(bal & ((1u << lane) - 1u));
                if (off < kMaxLocalSources) {
                    s_srcp[off] = p;
                    s_srcq0[off] = (Real)source_rate(F, G.n_src, s, pl.t0, area);
                    s_srcq1[off] = (Real)source_rate(F, G.n_src, s, pl.t1, area);
                } else {
                    atomicOr(&clk[slot_out].status, (unsigned)ST_TOO_MANY_LOCAL_SOURCES);
                }
            }
            __syncthreads();
            if (tid == 0) {
                int tot = s_nloc;
                for (int w = 0; w < NW; w++) tot += s_wcnt[w];
                s_nloc = tot < kMaxLocalSources ? tot : kMaxLocalSources;
            }
            __syncthreads();  // s_wcnt is rewritten by the next chunk
        }
    }
    __syncthreads();

    const Real rr0_u = LS.rr0, rr1_u = LS.rr1;
    const Real ev0 = LS.ev0, ev1 = LS.ev1;
    const Real *__restrict__ W = S.rainw;  // spatial rain factors (extension) or nullptr
    const int nloc = s_nloc;
    const Real pct_hi = GS.pct_hi, pct_lo = GS.pct_lo;
    const bool storm = F.rain_kind == RAIN_STORM;

    // ---- stage 1: face depths and velocities (cu:363-453) ------------------
    for (int idx = tid; idx < RN; idx += NT) {
        const int r = idx / RW, c = idx - (idx / RW) * RW;
        const int gi = I0 + r, gj = J0 + c;
        if (r >= 1) {
            Real hm;
            if (gi == rows) hm = s_h[idx - RW];
            else if (gi == 0) hm = s_h[idx];
            else hm = Real(0.50) * (s_h[idx] + s_h[idx - RW]);
            s_uu1[idx] = (hm >= T.ge_th) ? s_umo[idx] / hm : Real(0.00);
        }
        if (c >= 1) {
            Real hn;
            if (gj == cols) hn = s_h[idx - 1];
            else if (gj == 0) hn = s_h[idx];
            else hn = Real(0.50) * (s_h[idx] + s_h[idx - 1]);
            s_vv1[idx] = (hn >= T.ge_th) ? s_vno[idx] / hn : Real(0.0);
        }
    }
    __syncthreads();

    // ---- stage 2: new face discharges (cu:98-354) ---------------------------
    constexpr int FH = TH + 4, FW = TW + 4;  // rows/cols [2, TH+6) x [2, TW+6)
    for (int k = tid; k < FH * FW; k += NT) {
        const int r = 2 + k / FW, c = 2 + (k - (k / FW) * FW);
        const int p = r * RW + c;
        const int gi = I0 + r, gj = J0 + c;
        // x-face (gi, gj): between cells (gi-1, gj) "a" and (gi, gj) "b"
        Real qx = 0;
        if ((unsigned)gj < (unsigned)cols) {
            if (gi > 0 && gi < rows) {
                const int pa = p - RW;
                const Real hb = s_h[p], ha = s_h[pa];
                if (s_m[p] && s_m[pa] && ((ha >= T.gt_th) || (hb >= T.gt_th))) {
                    const Real zb = s_z[p], za = s_z[pa];
                    if (!dry_bed<Real>(T, g, ha, za, hb, zb, qx)) {
                        const Real hm = Real(0.50) * (hb + ha);
                        const Real u13 = g * hm * dt2dx * (hb + zb - ha - za);  // cu:166
                        const Real uu_s = s_uu1[p + RW], uu_c = s_uu1[p], uu_n = s_uu1[pa];
                        const Real mo_s = s_umo[p + RW], mo_c = s_umo[p], mo_n = s_umo[pa];
                        const Real u11uur = Real(0.50) * (uu_s + uu_c);
                        const Real u11uul = Real(0.50) * (uu_c + uu_n);
                        const Real umr = upwind<Real>(u11uur, mo_s, mo_c);
                        const Real uml = upwind_r<Real>(u11uul, mo_n, mo_c);
                        const Real u11 = dt2dx * (umr - uml);  // cu:176
                        Real u12;
                        if (gj == 0) {
                            u12 = 0;  // cu:178-180
                        } else {
                            const Real u12vvu = Real(0.50) * (s_vv1[p + 1] + s_vv1[pa + 1]);
                            const Real u12vvd = Real(0.50) * (s_vv1[p] + s_vv1[pa]);
                            const Real umu = upwind<Real>(u12vvu, s_umo[p + 1], mo_c);
                            const Real umd = upwind_r<Real>(u12vvd, s_umo[p - 1], mo_c);
                            u12 = dt2dy * (umu - umd);  // cu:189
                        }
                        const Real rn = has_n ? Real(0.5) * (s_n[p] + s_n[pa]) : manning;
                        Real ram = 0;
                        if (!(hm < T.gt_th) && rn != Real(0)) {  // cu:194-199: zero only when hm <= th
                            const Real vva = Real(0.250) * (s_vv1[p] + s_vv1[p + 1] + s_vv1[pa] + s_vv1[pa + 1]);
                            const Real sqx = RT<Real>::sqrt_(uu_c * uu_c + vva * vva);
                            ram = g * rn * rn * sqx / RT<Real>::pow_(hm);
                        }
                        qx = ((Real(1.00) - dt2 * ram * Real(0.50)) * mo_c + (-u11 - u12 - u13)) /
                             (Real(1.00) + dt2 * ram * Real(0.50));  // cu:203
                    }
                }
            } else if (gi == rows && G.south_open) {
                const int pa = p - RW;
                const Real ha = s_h[pa];
                qx = (s_m[pa] && ha >= T.gt_th) ? Real(0.5440) * ha * RT<Real>::sqrt_(g * ha) : Real(0);
            }
        }
        s_rum[p] = qx;
        // y-face (gi, gj): between cells (gi, gj-1) "a" and (gi, gj) "b"
        Real qy = 0;
        if ((unsigned)gi < (unsigned)rows && gj > 0 && gj < cols) {
            const int pa = p - 1;
            const Real hb = s_h[p], ha = s_h[pa];
            if (s_m[p] && s_m[pa] && ((ha >= T.gt_th) || (hb >= T.gt_th))) {
                const Real zb = s_z[p], za = s_z[pa];
                if (!dry_bed<Real>(T, g, ha, za, hb, zb, qy)) {
                    const Real hn = Real(0.50) * (hb + ha);
                    const Real v13 = g * hn * dt2dy * (hb + zb - ha - za);  // cu:283
                    const Real mo_c = s_vno[p];
                    Real v11;
                    if (gi == 0) {
                        v11 = 0;  // cu:289-291
                    } else {
                        const Real v11uur = Real(0.50) * (s_uu1[p + RW] + s_uu1[p + RW - 1]);
                        const Real v11uul = Real(0.50) * (s_uu1[p] + s_uu1[p - 1]);
                        const Real vnr = upwind<Real>(v11uur, s_vno[p + RW], mo_c);
                        const Real vnl = upwind_r<Real>(v11uul, s_vno[p - RW], mo_c);
                        v11 = dt2dx * (vnr - vnl);  // cu:300
                    }
                    const Real vv_c = s_vv1[p];
                    const Real v12vvu = Real(0.50) * (s_vv1[p + 1] + vv_c);
                    const Real v12vvd = Real(0.50) * (vv_c + s_vv1[p - 1]);
                    const Real vnu = upwind<Real>(v12vvu, s_vno[p + 1], mo_c);
                    const Real vnd = upwind_r<Real>(v12vvd, s_vno[p - 1], mo_c);
                    const Real v12 = dt2dy * (vnu - vnd);  // cu:307
                    const Real rn = has_n ? Real(0.5) * (s_n[p] + s_n[pa]) : manning;
                    Real ram = 0;
                    if (!(hn < T.gt_th) && rn != Real(0)) {  // cu:311-316: zero only when hn <= th
                        const Real uua = Real(0.250) * (s_uu1[p] + s_uu1[p + RW] + s_uu1[p - 1] + s_uu1[p + RW - 1]);
                        const Real sqy = RT<Real>::sqrt_(uua * uua + vv_c * vv_c);
                        ram = g * rn * rn * sqy / RT<Real>::pow_(hn);
                    }
                    qy = ((Real(1.00) - dt2 * ram * Real(0.50)) * mo_c + (-v11 - v12 - v13)) /
                         (Real(1.00) + dt2 * ram * Real(0.50));  // cu:320
                }
            }
        }
        s_rvn[p] = qy;
    }
    __syncthreads();

    // storm rain at a cell centre; the centre (sx, sy) is per launch
    const Real storm_amp = GS.storm_amp, storm_2s2 = GS.storm_2s2;
    auto storm_rate = [&](int gi, int gj, bool on, Real sx, Real sy) -> Real {
        if (!on) return Real(0);
        const Real x = ((Real)gj + Real(0.5)) * dx - sx;
        const Real y = ((Real)gi + Real(0.5)) * dy - sy;
        return storm_amp * RT<Real>::exp_(-(x * x + y * y) / storm_2s2);
    };
    const Real sx0 = LS.sx0, sy0 = LS.sy0, sx1 = LS.sx1, sy1 = LS.sy1;

    // ---- stage 3: provisional depth with forcing at t (cu:1278-1288) -------
    constexpr int PH = TH + 3, PW = TW + 3;  // rows/cols [2, TH+5) x [2, TW+5)
    for (int k = tid; k < PH * PW; k += NT) {
        const int r = 2 + k / PW, c = 2 + (k - (k / PW) * PW);
        const int p = r * RW + c;
        Real hv = 0;
        if (s_m[p]) {
            const Real ho = s_h[p];
            const bool hi = ho >= T.gt_evmin;
            const Real pct = hi ? pct_hi : pct_lo;
            const Real evapo = hi ? ev0 : Real(0.000);
            Real ql = 0;
            for (int q = 0; q < nloc; q++)
                if (s_srcp[q] == p) ql = s_srcq0[q];
            Real rr = storm ? storm_rate(I0 + r, J0 + c, pl.storm_on0, sx0, sy0) : rr0_u;
            if (W) rr = rr * W[(size_t)(I0 + r) * pitch + (J0 + c)];
            hv = ho - dt2 * ((s_rum[p + RW] - s_rum[p]) / dx + (s_rvn[p + 1] - s_rvn[p]) / dy - ql - rr * pct + evapo);
            hv = fmax(hv, Real(0.00));  // cu:657
        }
        s_hs[p] = hv;
    }
    __syncthreads();

    // ---- stage 4: dry-cell fix per face (cu:695-725) + final depth ----------
    // corrected x-face at p: zero if it drains a dry cell
    auto fix_x = [&](int p) -> Real {
        const Real q = s_rum[p];
        if (q > Real(0) && s_m[p - RW] && s_hs[p - RW] < T.ge_th) return Real(0);
        if (q < Real(0) && s_m[p] && s_hs[p] < T.ge_th) return Real(0);
        return q;
    };
    auto fix_y = [&](int p) -> Real {
        const Real q = s_rvn[p];
        if (q > Real(0) && s_m[p - 1] && s_hs[p - 1] < T.ge_th) return Real(0);
        if (q < Real(0) && s_m[p] && s_hs[p] < T.ge_th) return Real(0);
        return q;
    };

    // per-thread partials in the working precision; FP64 from the warp sums on
    Real b_rain = 0, b_src = 0, b_ev = 0, b_out = 0, b_clamp = 0;
    bool bad = false;
    constexpr int OH = TH + 1, OW = TW + 1;  // rows/cols [3, TH+4) x [3, TW+4)
    for (int k = tid; k < OH * OW; k += NT) {
        const int r = 3 + k / OW, c = 3 + (k - (k / OW) * OW);
        const int p = r * RW + c;
        const int gi = I0 + r, gj = J0 + c;
        const Real un = fix_x(p), us = fix_x(p + RW), vw = fix_y(p), ve = fix_y(p + 1);
        Real hv = 0, hraw = 0;
        const bool act = s_m[p] != 0;
        Real ql = 0, rr = 0, pct = 0, evapo = 0;
        if (act) {
            const Real ho = s_h[p];
            const bool hi = ho >= T.gt_evmin;
            pct = hi ? pct_hi : pct_lo;
            evapo = hi ? ev1 : Real(0.000);
            for (int q = 0; q < nloc; q++)
                if (s_srcp[q] == p) ql = s_srcq1[q];
            rr = storm ? storm_rate(gi, gj, pl.storm_on1, sx1, sy1) : rr1_u;
            if (W) rr = rr * W[(size_t)gi * pitch + gj];
            hraw = ho - dt2 * ((us - un) / dx + (ve - vw) / dy - ql - rr * pct + evapo);
            hv = fmax(hraw, Real(0.00));
        }
        s_h[p] = hv;  // the new depth; only this thread reads s_h[p] in this stage
        s_umo[p] = un;
        s_vno[p] = vw;
        if (r == TH + 3) s_umo[p + RW] = us;
        if (c == TW + 3) s_vno[p + 1] = ve;
        const bool core = r >= HN && c >= HN && r < TH + HN && c < TW + HN && gi < rows && gj < cols;
        if (core) {
            const size_t gp = (size_t)gi * pitch + gj;
            Hout[gp] = hv;
            Uout[gp] = un;
            Vout[gp] = vw;
            if (gi == rows - 1) {
                Uout[gp + pitch] = us;
                b_out += us;
            }
            if (act) {
                b_rain += rr * pct;
                b_src += ql;
                b_ev += evapo;
                if (hraw < Real(0)) b_clamp -= hraw;
            }
            if (!RT<Real>::finite_(hv) || !RT<Real>::finite_(un) || !RT<Real>::finite_(vw)) bad = true;
        }
    }
    __syncthreads();

    // ---- stage 5: CFL bound of the new state over the owned faces ----------
    Real cm = 0;
    for (int k = tid; k < TH * TW; k += NT) {
        const int r = HN + k / TW, c = HN + (k - (k / TW) * TW);
        const int p = r * RW + c;
        const int gi = I0 + r, gj = J0 + c;
        if (gi >= rows || gj >= cols) continue;
        if (gi > 0 && s_m[p] && s_m[p - RW]) {
            const Real hm = Real(0.50) * (s_h[p] + s_h[p - RW]);
            if (hm >= T.ge_th) {
                const Real v = fabs(s_umo[p] / hm) + RT<Real>::sqrt_(g * hm);
                cm = fmax(cm, v);
            }
        }
        if (gi == rows - 1 && G.south_open && s_m[p]) {
            const Real hm = s_h[p];
            if (hm >= T.ge_th) {
                const Real v = fabs(s_umo[p + RW] / hm) + RT<Real>::sqrt_(g * hm);
                cm = fmax(cm, v);
            }
        }
        if (gj > 0 && s_m[p] && s_m[p - 1]) {
            const Real hn = Real(0.50) * (s_h[p] + s_h[p - 1]);
            if (hn >= T.ge_th) {
                const Real v = fabs(s_vno[p] / hn) + RT<Real>::sqrt_(g * hn);
                cm = fmax(cm, v);
            }
        }
    }

    // ---- block reductions (working precision), one atomic per quantity ----
    Real vals[B_N + 1] = {b_rain, b_src, b_ev, b_out, b_clamp, cm};
    const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
    for (int q = 0; q < B_N; q++) {
        Real v = vals[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        vals[q] = v;
    }
    {
        Real v = vals[B_N];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        vals[B_N] = v;
    }
    const bool any_bad = __syncthreads_or(bad);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q <= B_N; q++) s_red[wid][q] = vals[q];
    }
    __syncthreads();
    if (tid >= 32) return;
    if (tid == 0) {
        Real acc[B_N + 1];
#pragma unroll
        for (int q = 0; q <= B_N; q++) acc[q] = s_red[0][q];
        for (int w = 1; w < NW; w++) {
#pragma unroll
            for (int q = 0; q < B_N; q++) acc[q] += s_red[w][q];
            acc[B_N] = fmax(acc[B_N], s_red[w][B_N]);
        }
        const double area = G.dx * G.dy;
        const double scale = pl.d.dt2 * area;
        double v[B_N];
        v[B_RAIN] = (double)acc[B_RAIN] * scale;
        v[B_SRC] = (double)acc[B_SRC] * scale;
        v[B_EV] = (double)acc[B_EV] * scale;
        v[B_OUT] = (double)acc[B_OUT] * pl.d.dt2 * G.dy;
        v[B_CLAMP] = (double)acc[B_CLAMP] * area;
        accumulate_slot(clk[slot_out], blockIdx.x % kBuckets, v, (double)acc[B_N], any_bad);
    }
    finish_cta_warp(lane, ci, clk[slot_out], clk[slot_nx], pl, *ctl, G, F);
}

// Plans the launch that will read slot `slot` (used when a run starts or its
// control changes).  One warp.
static __global__ void plan_kernel(const GridDesc G, const ForcingDesc F, Clock *__restrict__ clk,
                            const Control *__restrict__ ctl, const int slot) {
    Clock &c = clk[slot];
    const Plan p = make_plan_warp((int)threadIdx.x, c.t, c.cmax_bits, c.steps, *ctl, G, F);
    if (threadIdx.x == 0) c.plan = p;
}

}  // namespace sw2d
