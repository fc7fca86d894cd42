// sw2d_pipe.cuh -- the FP32 streaming kernel with several iterations per
// launch (temporal blocking without recomputed halos), for the fixed time
// step.
//
// Under the reference's time-step rule -- a constant half step dt (cu:790,
// cu:808), looping while t + dt <= t_end (cu:1256) -- every iteration's step,
// time and forcing are known before a launch starts, so only the cells
// around a unit couple its iterations to the rest of the grid.  One
// cooperative launch runs K iterations:
//
//   * pipe_plan_kernel (one CTA) writes the K plans -- the time recurrence
//     t <- (t + dt) + dt (cu:1297, cu:1335) and the forcing at t and t + dt,
//     formed by the same operations as in the one-iteration launches -- and
//     the number of leading iterations that run, and clears the progress
//     counters;
//   * stream_pipe_kernel: every warp keeps one unit (column tile x strip)
//     for all K iterations.  Its window reads only cells of the (up to
//     eight) units around it -- rows R0 - 7 .. R1 + 2 and columns gj0 - 1 ..
//     gj0 + 32 lie within one strip and one column tile on either side once
//     strips have kPipeMinStrip rows -- and the buffer it writes in
//     iteration j is the one they read in iteration j - 1.  So before
//     iteration j > 0 it waits until the units of the strip above and its
//     own strip have finished iteration j - 1, and the units of the strip
//     below have passed their first rows of it: of those it reads only their
//     first three output rows, and they read the rows above their strip
//     before they write these.  Each unit publishes two counts with release
//     stores after the writes they cover -- iterations finished, and
//     iterations whose first rows are done (stream_unit, PIPE); the waits
//     read them with acquire loads, and the state is read past L1.
//
// Waiting for the strip below only up to its first rows matters: the warp
// scheduler favours older warps, so units of later strips (launched later)
// run slower, and a wait for their whole iteration would hold every strip
// to the pace of the last one.
//
// A unit that finishes early starts its next iteration as soon as its
// neighbours allow, instead of idling until the slowest unit of the grid
// has finished and the last CTA has planned the next launch: the grid-wide
// drain of every iteration (the tail of the slowest SM, the finalising CTA,
// the launch gap) is paid once per K iterations.
//
// The launch is cooperative, so every unit is resident and every wait ends;
// each wait is bounded all the same (kPipeWaitPolls, about a second): a wait
// that gives up raises ST_PIPE_TIMEOUT, ends that warp's iterations and sets
// the launch's abort word, which ends every other warp's wait at once.  The
// host sizes strips so that one wave of resident warps holds every unit.
//
// Budgets: each warp adds its per-iteration sums, scaled in FP64, in shared
// memory; per CTA they go to the clock slot's buckets once per launch, and
// the last CTA finalises the slot with the launch's iteration count.  The
// state after a launch is bit for bit what K one-iteration launches leave;
// the budgets are the same terms added in another order.
#pragma once

#include "sw2d_stream.cuh"

namespace sw2d {

constexpr int kPipeWaitPolls = 1 << 20;  // polls of one wait (each a load and a ~100 ns sleep: about a second)
constexpr int kPipeMinStrip = 8;         // rows per strip for the neighbour set above
constexpr int kPipeMaxIters = 1024;      // iterations per launch (one plan per thread)

struct PipeDesc {
    const Plan *plans;  // plans of the launch's iterations
    unsigned *words;    // [0]: iterations the launch runs, [1]: abort (a wait gave up)
    unsigned *flags;    // [u]: iterations unit u finished in this launch; [units + u]: iterations
                        // whose first output rows it has written
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_relaxed_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// True once every unit watched by a lane of the warp (nb >= 0) has finished
// `need` iterations; false if the wait gave up or another warp's did (lane 9
// watches the abort word).
__device__ __forceinline__ bool wait_units(const unsigned *flags, const unsigned *abort_word, int nb,
                                           unsigned need, int lane) {
    bool ok = nb < 0;
    for (int it = 0; it < kPipeWaitPolls; it++) {
        if (!ok) ok = ld_acquire_gpu(flags + nb) >= need;
        if (__all_sync(0xffffffffu, ok)) return true;
        const bool stop = lane == 9 && ld_relaxed_gpu(abort_word) != 0u;
        if (__any_sync(0xffffffffu, stop)) return false;
        __nanosleep(100);
    }
    return false;
}

// Plans of the iterations of one pipelined launch.  Thread j carries the
// slot's clock through j iterations as the finalising CTAs of one-iteration
// launches do and plans iteration j (make_plan_serial: the operations of
// make_plan_warp); the launch runs the leading iterations whose plan runs.
static __global__ void pipe_plan_kernel(const GridDesc G, const ForcingDesc F, const Clock *__restrict__ clk,
                                        const Control *__restrict__ ctl, const int slot, Plan *__restrict__ plans,
                                        unsigned *__restrict__ words, unsigned *__restrict__ flags, const int units,
                                        const int K) {
    const int j = threadIdx.x;
    for (int u = j; u < 2 * units; u += blockDim.x) flags[u] = 0u;
    if (j == 0) words[1] = 0u;
    __shared__ int s_count;
    if (j == 0) s_count = K;
    __syncthreads();
    if (j < K) {
        const Clock &c = clk[slot];
        double t = c.t;
        long long steps = c.steps;
        bool ok = true;
        for (int k = 0; k < j; k++) {
            double dt = 0.0;
            if (!decide_step(t, 0.0, steps, *ctl, G, &dt)) {
                ok = false;
                break;
            }
            t = (t + dt) + dt;
            steps++;
        }
        Plan p = make_plan_serial(t, c.cmax_bits, steps, *ctl, G, F);
        if (!ok) p.run = 0;
        plans[j] = p;
        if (!p.run) atomicMin(&s_count, j);
    }
    __syncthreads();
    if (j == 0) words[0] = (unsigned)s_count;
}

template <int NWARP, int MINB, int UNR, bool RAINW, bool GEN>
__global__ void __launch_bounds__(NWARP * 32, MINB)
    stream_pipe_kernel(const GridDesc G, const ForcingDesc F, const StateBufs<float> S, const Thr<float> T,
                       Clock *__restrict__ clk, const Control *__restrict__ ctl, const int slot,
                       const StreamShape SH, const PipeDesc P) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int slot_out = slot == 2 ? 0 : slot + 1;
    const int slot_nx = slot == 0 ? 2 : slot - 1;
    const Clock &ci = clk[slot];
    const int K = (int)P.words[0];
    if (K <= 0) {
        if (blockIdx.x == 0 && tid == 0) carry_slot(ci, clk[slot_out], clk[slot_nx]);
        return;
    }

    __shared__ int s_sr[NWARP][kStreamMaxSrc], s_sc[NWARP][kStreamMaxSrc];
    __shared__ float s_q0[NWARP][kStreamMaxSrc], s_q1[NWARP][kStreamMaxSrc];
    __shared__ double s_acc[NWARP][B_N];
    __shared__ float s_cm[NWARP];
    __shared__ unsigned s_st[NWARP];  // bit 0: non-finite, 1: too many local sources, 2: a wait gave up
    if (lane == 0) {
        for (int q = 0; q < B_N; q++) s_acc[wid][q] = 0.0;
        s_cm[wid] = 0.f;
        s_st[wid] = 0u;
    }
    __syncwarp();

    // the unit broadcast from lane 0, as in stream_step_body: its rows and
    // everything derived from them stay in uniform registers
    const int w_unit = __shfl_sync(0xffffffffu, (int)blockIdx.x * NWARP + wid, 0);
    if (w_unit < SH.units) {
        // units are handed to warps in a scattered order, so that the warps
        // sharing an SM hold units from all over the grid: the SMs then carry
        // the same work (edge tiles, the longer strips) and the scheduler's
        // preference for older warps does not fall on one part of the grid
        const int unit = __shfl_sync(0xffffffffu, unit_of_warp(SH, w_unit), 0);
        const int ct = unit % SH.tiles_w, rs = unit / SH.tiles_w;
        const int nstrips = SH.strips;
        int r0, r1;
        strip_rows(G.rows, SH.strips, SH.skew, rs, r0, r1);
        r0 = __shfl_sync(0xffffffffu, r0, 0);  // the strip's rows, warp-uniform
        r1 = __shfl_sync(0xffffffffu, r1, 0);
        // lanes 0-8 but 4 watch the unit at (strip rs + lane/3 - 1, tile ct +
        // lane%3 - 1): its count of finished iterations, or for the strip
        // below (lanes 6-8) its count of iterations with the first rows done
        int nb = -1;
        if (lane < 9 && lane != 4) {
            const int r2 = rs + lane / 3 - 1, c2 = ct + lane % 3 - 1;
            if (r2 >= 0 && r2 < nstrips && c2 >= 0 && c2 < SH.tiles_w)
                nb = r2 * SH.tiles_w + c2 + (lane >= 6 ? SH.units : 0);
        }
        const double area = G.dx * G.dy;
        for (int j = 0; j < K; j++) {
            if (j > 0) {
                const bool ok = wait_units(P.flags, P.words + 1, nb, (unsigned)j, lane);
                __syncwarp();  // the acquire of lanes 0-8 orders every lane's reads below
                if (!ok) {
                    if (lane == 0) {
                        s_st[wid] |= 4u;
                        atomicExch(P.words + 1, 1u);  // end every other wait of the launch
                    }
                    break;
                }
            }
            const Plan &pl = P.plans[j];
            const int b = ci.buf ^ (j & 1);
            StreamView V;
            V.rows = G.rows;
            V.cols = G.cols;
            V.pitch = G.pitch;
            V.south_open = G.south_open;
            V.Hin = S.h[b];
            V.Uin = S.um[b];
            V.Vin = S.vn[b];
            V.DZX = S.dzx;
            V.DZY = S.dzy;
            V.Rin = S.hr[b];
            V.Rout = S.hr[1 - b];
            V.Nin = S.nman;
            V.Min = S.mask;
            V.Win = S.rainw;
            V.Hout = S.h[1 - b];
            V.Uout = S.um[1 - b];
            V.Vout = S.vn[1 - b];
            V.GS = G.sf;
            V.T = T;
            V.LS = pl.f;
            V.storm = F.rain_kind == RAIN_STORM;
            V.on0 = pl.storm_on0;
            V.on1 = pl.storm_on1;
            V.n_src = G.n_src;
            V.F = &F;
            V.t0 = pl.t0;
            V.t1 = pl.t1;
            V.dx = G.dx;
            V.dy = G.dy;
            StreamAcc A;
            A.rain = A.src = A.ev = A.out = A.clamp = A.cm = 0.f;
            A.bad = A.too_many_sources = false;
            stream_unit<UNR, RAINW, GEN, false, true>(V, ct, r0, r1, lane, s_sr[wid], s_sc[wid], s_q0[wid],
                                                      s_q1[wid], A, nullptr, 0, nullptr, nullptr,
                                                      P.flags + SH.units + unit, (unsigned)(j + 1));
            warp_reduce_acc(A);
            if (lane == 0) {
                const double scale = pl.d.dt2 * area;
                s_acc[wid][B_RAIN] += (double)A.rain * scale;
                s_acc[wid][B_SRC] += (double)A.src * scale;
                s_acc[wid][B_EV] += (double)A.ev * scale;
                s_acc[wid][B_OUT] += (double)A.out * pl.d.dt2 * G.dy;
                s_acc[wid][B_CLAMP] += (double)A.clamp * area;
                s_cm[wid] = A.cm;  // the CFL bound of the launch's final state
                s_st[wid] |= (A.bad ? 1u : 0u) | (A.too_many_sources ? 2u : 0u);
            }
            __syncwarp();  // every lane's stores of this iteration come before the release
            if (lane == 0) st_release_gpu(P.flags + unit, (unsigned)(j + 1));
        }
    }

    // ---- per CTA: the launch's budget sums, CFL bound and status bits ----
    __syncthreads();
    if (wid != 0) return;
    if (lane == 0) {
        double v[B_N];
        for (int q = 0; q < B_N; q++) v[q] = 0.0;
        float cmb = 0.f;
        unsigned st = 0u;
        for (int w = 0; w < NWARP; w++) {
            for (int q = 0; q < B_N; q++) v[q] += s_acc[w][q];
            cmb = fmaxf(cmb, s_cm[w]);
            st |= s_st[w];
        }
        accumulate_slot(clk[slot_out], blockIdx.x % kBuckets, v, (double)cmb, (st & 1u) != 0u);
        if (st & 2u) atomicOr(&clk[slot_out].status, (unsigned)ST_TOO_MANY_LOCAL_SOURCES);
        if (st & 4u) atomicOr(&clk[slot_out].status, (unsigned)ST_PIPE_TIMEOUT);
    }
    finish_cta_warp(lane, ci, clk[slot_out], clk[slot_nx], P.plans[K - 1], *ctl, G, F, K);
}

}  // namespace sw2d
