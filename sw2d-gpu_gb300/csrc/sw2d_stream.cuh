// sw2d_stream.cuh -- FP32 warp-streaming step kernel (one scenario).
//
// The same iteration as step_kernel (one iteration of the reference loop
// SW2D-GPU_linux/src/SW2D-GPU.cu:1256-1336), organised for the FP32 path's
// instruction budget instead of for FP64 reuse:
//
//   * one warp owns 32 adjacent columns -- 27 output columns plus 3 halo
//     columns on the west and 2 on the east, the lateral dependency radius
//     of one iteration (shortened by loading the neighbours' depths and
//     discharges at the window's edges) -- and marches down a strip of rows
//     (stream_unit in sw2d_stream_unit.cuh);
//   * each row read from HBM (h, the face bed differences dzx and dzy, n,
//     mask, um, vn and the depth remainder; one coalesced line per field and
//     warp) feeds a 3-row register pipeline
//         row r    : face depths and velocities uu1/vv1        (cu:363-453)
//         row r-1  : new face discharges, momentum + dry bed   (cu:98-354)
//         row r-2  : provisional depth, forcing at t           (cu:603-665)
//         row r-3  : dry-cell fix per face (cu:695-725), final depth with
//                    forcing at t+dt, CFL bound of the owned faces
//     so every quantity is computed once per cell and row, in registers;
//   * west/east neighbours come from warp shuffles, except the neighbours'
//     depths and y discharge that each lane loads itself (they make the
//     window's edge lanes exact); an upwinded flux shared by two faces is
//     formed once (the next row's, or the neighbour lane's, by a shuffle);
//     there is no shared-memory tile and no block-wide barrier inside the
//     row loop;
//   * the next row's loads are issued before the current row's arithmetic.
//
// Budgets and the CFL bound are reduced per warp and then per CTA; the last
// CTA of the launch finalises the clock slot's time and plan, the first to
// finish folds the budgets of the slot the launch read
// (finish_cta_deferred_warp).  Launches
// are programmatic dependents of the previous iteration (launch_stream_step):
// the next grid's CTAs are scheduled while this one drains and finalises,
// and wait for its completion before they read anything.
#pragma once

#include "sw2d_stream_unit.cuh"

namespace sw2d {

struct StreamShape {
    int tiles_w;  // column tiles of kStreamOut columns
    int strips;   // strips per column tile
    int units;    // tiles_w * strips
    int perm;     // warp w runs unit (w * perm) % units (perm coprime with units; 1 = in order)
    int skew;     // percent by which strip heights fall from the first strip to the last (0 = even)
    int pad[3];
};

// First row of strip k when strip heights follow the density
// 1 + (skew/100)(1/2 - x) over x = k / strips: the boundary rounded to the
// nearest row, in exact integer arithmetic.
__device__ __forceinline__ int strip_start(int rows, int strips, int skew, int k) {
    const long long R = rows, n = strips, kk = k;
    return (int)((R * kk * 200 * n + skew * R * kk * (n - kk) + 100 * n * n) / (200 * n * n));
}

// Rows [r0, r1) of strip rs of `strips`.  skew == 0: heights differ by at
// most one row (the first rows % strips are the longer).  skew > 0: heights
// fall linearly from (1 + skew/200) to (1 - skew/200) of the mean, so that
// the strips of the CTAs launched first -- which the warp scheduler favours
// as the older warps -- carry more rows, and all warps of an SM finish at
// about the same time.
__device__ __forceinline__ void strip_rows(int rows, int strips, int skew, int rs, int &r0, int &r1) {
    if (skew == 0) {
        const int q = rows / strips, rem = rows - q * strips;
        r0 = rs * q + min(rs, rem);
        r1 = r0 + q + (rs < rem ? 1 : 0);
    } else {
        r0 = strip_start(rows, strips, skew, rs);
        r1 = strip_start(rows, strips, skew, rs + 1);
    }
}

// The unit warp w runs.
__device__ __forceinline__ int unit_of_warp(const StreamShape &SH, int w) {
    return SH.perm == 1 ? w : (int)(((long long)w * SH.perm) % SH.units);
}

// The body of one launch.  RAINW: per-cell rain factors; GEN: moving storm
// and point sources (the launcher picks the build from the handle's
// forcing); TMA: rows staged in shared memory by TMA (M: the planes' tensor
// maps, smem: kTmaStages stages per warp).
template <int NWARP, int MINB, int UNR, bool RAINW, bool GEN, bool TMA>
__device__ __forceinline__ void stream_step_body(const GridDesc &G, const ForcingDesc &F, const StateBufs<float> &S,
                                                 const Thr<float> &T, Clock *__restrict__ clk,
                                                 const Control *__restrict__ ctl, const int slot,
                                                 const StreamShape &SH, const TmaMaps *M, unsigned char *smem) {
    // Launched as a programmatic dependent of the previous iteration: wait
    // until that grid has completed and its writes are visible, then let the
    // next iteration's grid be scheduled (its CTAs wait the same way)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int slot_out = slot == 2 ? 0 : slot + 1;
    const int slot_nx = slot == 0 ? 2 : slot - 1;
    const Clock &ci = clk[slot];
    if (!ci.plan.run) {
        if (blockIdx.x == 0 && wid == 0) carry_slot_deferred_warp(lane, clk, slot, slot_out, slot_nx);
        return;
    }

    __shared__ int s_sr[NWARP][kStreamMaxSrc], s_sc[NWARP][kStreamMaxSrc];
    __shared__ float s_q0[NWARP][kStreamMaxSrc], s_q1[NWARP][kStreamMaxSrc];
    __shared__ float s_red[NWARP][B_N + 1];
    __shared__ int s_bad[NWARP], s_many[NWARP];

    StreamAcc A;
    A.rain = A.src = A.ev = A.out = A.clamp = A.cm = 0.f;
    A.bad = A.too_many_sources = false;
    // broadcast from lane 0: the compiler then knows the unit, its rows and
    // every quantity derived from them to be warp-uniform and keeps them in
    // uniform registers (measured 7-8 % faster than the plain expression)
    const int w_unit = __shfl_sync(0xffffffffu, (int)blockIdx.x * NWARP + wid, 0);
    const int unit = __shfl_sync(0xffffffffu, w_unit < SH.units ? unit_of_warp(SH, w_unit) : w_unit, 0);
    __shared__ __align__(8) unsigned long long s_bar[TMA ? NWARP : 1][kTmaStages];
    if (TMA && lane == 0) {
        for (int k = 0; k < kTmaStages; k++) mbar_init(&s_bar[wid][k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (TMA) __syncwarp();
    if (unit < SH.units) {
        StreamView V;
        const int b = ci.buf;
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
        V.LS = ci.plan.f;
        V.storm = F.rain_kind == RAIN_STORM;
        V.on0 = ci.plan.storm_on0;
        V.on1 = ci.plan.storm_on1;
        V.n_src = G.n_src;
        V.F = &F;
        V.t0 = ci.plan.t0;
        V.t1 = ci.plan.t1;
        V.dx = G.dx;
        V.dy = G.dy;
        int r0, r1;
        strip_rows(G.rows, SH.strips, SH.skew, unit / SH.tiles_w, r0, r1);
        r0 = __shfl_sync(0xffffffffu, r0, 0);  // the strip's rows, warp-uniform (see above)
        r1 = __shfl_sync(0xffffffffu, r1, 0);
        stream_unit<UNR, RAINW, GEN, TMA>(V, unit % SH.tiles_w, r0, r1, lane, s_sr[wid],
                                          s_sc[wid], s_q0[wid], s_q1[wid], A, M, b,
                                          TMA ? smem + wid * kTmaStages * kTmaStageBytes : nullptr,
                                          TMA ? s_bar[wid] : nullptr);
    }
    if (TMA) {  // every copy issued was waited for: the barriers can go
        __syncwarp();
        if (lane == 0)
            for (int k = 0; k < kTmaStages; k++) mbar_inval(&s_bar[TMA ? wid : 0][k]);
    }

    // ---- warp, then CTA reductions; one thread accumulates and finishes ----
    warp_reduce_acc(A);
    if (lane == 0) {
        s_red[wid][B_RAIN] = A.rain;
        s_red[wid][B_SRC] = A.src;
        s_red[wid][B_EV] = A.ev;
        s_red[wid][B_OUT] = A.out;
        s_red[wid][B_CLAMP] = A.clamp;
        s_red[wid][B_N] = A.cm;
        s_bad[wid] = A.bad;
        s_many[wid] = A.too_many_sources;
    }
    __syncthreads();
    if (wid != 0) return;
    if (lane == 0) {
        double acc[B_N] = {0, 0, 0, 0, 0};
        float cmb = 0.f;
        bool anybad = false, many = false;
        for (int w = 0; w < NWARP; w++) {
            for (int q = 0; q < B_N; q++) acc[q] += (double)s_red[w][q];
            cmb = fmaxf(cmb, s_red[w][B_N]);
            anybad |= s_bad[w] != 0;
            many |= s_many[w] != 0;
        }
        const double area = G.dx * G.dy, scale = ci.plan.d.dt2 * area;
        double v[B_N];
        v[B_RAIN] = acc[B_RAIN] * scale;
        v[B_SRC] = acc[B_SRC] * scale;
        v[B_EV] = acc[B_EV] * scale;
        v[B_OUT] = acc[B_OUT] * ci.plan.d.dt2 * G.dy;
        v[B_CLAMP] = acc[B_CLAMP] * area;
        accumulate_slot(clk[slot_out], blockIdx.x % kBuckets, v, (double)cmb, anybad);
        if (many) atomicOr(&clk[slot_out].status, (unsigned)ST_TOO_MANY_LOCAL_SOURCES);
    }
    finish_cta_deferred_warp(lane, clk, slot, slot_out, slot_nx, ci.plan, *ctl, G, F);
}

template <int NWARP, int MINB, int UNR, bool RAINW, bool GEN>
__global__ void __launch_bounds__(NWARP * 32, MINB)
    stream_step_kernel(const GridDesc G, const ForcingDesc F, const StateBufs<float> S, const Thr<float> T,
                       Clock *__restrict__ clk, const Control *__restrict__ ctl, const int slot,
                       const StreamShape SH) {
    stream_step_body<NWARP, MINB, UNR, RAINW, GEN, false>(G, F, S, T, clk, ctl, slot, SH, nullptr, nullptr);
}

// The build that stages rows in shared memory by TMA (uniform forcing only):
// kept as a measured alternative; the row copies cost more issue slots than
// the loads they replace in this per-warp pipeline.
template <int NWARP, int MINB, int UNR>
__global__ void __launch_bounds__(NWARP * 32, MINB)
    stream_step_tma_kernel(const GridDesc G, const ForcingDesc F, const StateBufs<float> S, const Thr<float> T,
                           Clock *__restrict__ clk, const Control *__restrict__ ctl, const int slot,
                           const StreamShape SH, const __grid_constant__ TmaMaps M) {
    extern __shared__ __align__(1024) unsigned char s_stage[];
    stream_step_body<NWARP, MINB, UNR, false, false, true>(G, F, S, T, clk, ctl, slot, SH, &M, s_stage);
}

}  // namespace sw2d
