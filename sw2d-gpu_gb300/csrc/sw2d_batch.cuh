// sw2d_batch.cuh -- many scenarios of uneven size advanced by one persistent
// FP32 launch per iteration.
//
// Each scenario keeps its own state, static fields, forcing, CFL time step
// and clock (three rotating slots, as a single-scenario handle).  The work of
// one launch is the list of (scenario, column tile, row strip) units of every
// scenario in the batch; a fixed grid of CTAs pulls units from a queue head
// (one atomic per unit), so scenarios of 64 x 64 and 2048 x 2048 cells share
// the GPU without load imbalance.  A scenario's units take a ticket when they
// finish; the last one finalises that scenario's clock slot (time, budgets,
// CFL bound, the plan of its next iteration) -- no warp ever waits.
//
// The unit table, its length and the scenario descriptors live in device
// memory, so the CUDA graph of launches stays valid while scenarios are
// admitted and retired between replays.  A scenario whose plan says "stop"
// (end time reached) costs one queue entry per unit and launch until it is
// retired.
#pragma once

#include "sw2d_stream_unit.cuh"

namespace sw2d {

// Compact per-scenario status for the host, written by the finaliser.
struct ScenarioStatus {
    double t;
    long long steps;
    int running;     // the next iteration will run (end time not reached)
    int nonfinite;
    unsigned status;
    int pad;
};

struct ScenarioDev {
    GridDesc G;
    ForcingDesc F;
    Thr<float> T;
    Control ctl;
    float *h[2], *um[2], *vn[2], *hr[2];  // hr: depth remainders (compensated depth)
    const float *z, *dzx, *dzy, *nman;  // elevation, bed differences across faces, Manning n
    const uint8_t *mask;
    Clock *clk;                // three slots
    ScenarioStatus *status;    // this scenario's entry of the batch status array
    int tiles_w, strip_h, nunits, pad;
};

struct BatchHeader {
    int n_units;               // length of the unit table
    int pad;
    unsigned int head[3];      // queue heads, one per launch parity
    unsigned int pad2;
};

struct BatchDev {
    ScenarioDev *scen;
    const int2 *units;         // (scenario slot, unit index within the scenario)
    BatchHeader *hdr;
};

__device__ inline void write_status(const Clock &c, ScenarioStatus *st) {
    st->t = c.t;
    st->steps = c.steps;
    st->running = c.plan.run;
    st->nonfinite = (int)c.nonfinite;
    st->status = c.status;
}

template <int NWARP, int MINB, int UNR>
__global__ void __launch_bounds__(NWARP * 32, MINB) batch_step_kernel(const BatchDev B, const int slot) {
    // Launched as a programmatic dependent of the previous iteration: wait
    // until that grid has completed and its writes are visible (the queue
    // head, every scenario's state and clock), then let the next iteration's
    // grid be scheduled; its CTAs wait here the same way
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    __shared__ int s_sr[NWARP][kStreamMaxSrc], s_sc[NWARP][kStreamMaxSrc];
    __shared__ float s_q0[NWARP][kStreamMaxSrc], s_q1[NWARP][kStreamMaxSrc];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int slot_out = slot == 2 ? 0 : slot + 1;
    const int slot_nx = slot == 0 ? 2 : slot - 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) B.hdr->head[slot_out] = 0u;  // queue of the next launch
    const int n_units = B.hdr->n_units;
    // with fewer units than warps, the warps past the unit count would only
    // find the queue empty: the first n_units warps pull every unit
    if ((int)blockIdx.x * NWARP + wid >= n_units) return;
    for (;;) {
        unsigned u = 0;
        if (lane == 0) u = atomicAdd(&B.hdr->head[slot], 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= (unsigned)n_units) break;
        const int2 ue = B.units[u];
        const ScenarioDev &S = B.scen[ue.x];
        const Clock &ci = S.clk[slot];
        const int run = ci.plan.run;
        if (run) {
            StreamView V;
            const int b = ci.buf;
            V.rows = S.G.rows;
            V.cols = S.G.cols;
            V.pitch = S.G.pitch;
            V.south_open = S.G.south_open;
            V.Hin = S.h[b];
            V.Uin = S.um[b];
            V.Vin = S.vn[b];
            V.DZX = S.dzx;
            V.DZY = S.dzy;
            V.Rin = S.hr[b];
            V.Rout = S.hr[1 - b];
            V.Nin = S.nman;
            V.Min = S.mask;
            V.Win = nullptr;  // batched scenarios rain uniformly
            V.Hout = S.h[1 - b];
            V.Uout = S.um[1 - b];
            V.Vout = S.vn[1 - b];
            V.GS = S.G.sf;
            V.T = S.T;
            V.LS = ci.plan.f;
            V.storm = S.F.rain_kind == RAIN_STORM;
            V.on0 = ci.plan.storm_on0;
            V.on1 = ci.plan.storm_on1;
            V.n_src = S.G.n_src;
            V.F = &S.F;
            V.t0 = ci.plan.t0;
            V.t1 = ci.plan.t1;
            V.dx = S.G.dx;
            V.dy = S.G.dy;
            StreamAcc A;
            A.rain = A.src = A.ev = A.out = A.clamp = A.cm = 0.f;
            A.bad = A.too_many_sources = false;
            const int ct = ue.y % S.tiles_w, rs = ue.y / S.tiles_w;
            // batched scenarios take neither a storm nor point sources nor rain
            // factors (sw2d_batch_add accepts none), so the uniform-forcing unit
            const int r0 = rs * S.strip_h;
            stream_unit<UNR, false, false>(V, ct, r0, min(r0 + S.strip_h, V.rows), lane, s_sr[wid], s_sc[wid],
                                           s_q0[wid], s_q1[wid], A);
            warp_reduce_acc(A);
            if (lane == 0) {
                const double area = S.G.dx * S.G.dy, scale = ci.plan.d.dt2 * area;
                double v[B_N];
                v[B_RAIN] = (double)A.rain * scale;
                v[B_SRC] = (double)A.src * scale;
                v[B_EV] = (double)A.ev * scale;
                v[B_OUT] = (double)A.out * ci.plan.d.dt2 * S.G.dy;
                v[B_CLAMP] = (double)A.clamp * area;
                accumulate_slot(S.clk[slot_out], ue.y % kBuckets, v, (double)A.cm, A.bad);
                if (A.too_many_sources) atomicOr(&S.clk[slot_out].status, (unsigned)ST_TOO_MANY_LOCAL_SOURCES);
            }
        }
        unsigned ticket = 0u;
        if (lane == 0) {
            __threadfence();
            ticket = atomicAdd(&S.clk[slot_out].done_blocks, 1u);
        }
        ticket = __shfl_sync(0xffffffffu, ticket, 0);
        if (ticket == (unsigned)S.nunits - 1u) {  // the scenario's last unit: the whole warp finalises
            __threadfence();
            if (run) finalize_slot_warp(lane, ci, S.clk[slot_out], S.clk[slot_nx], ci.plan, S.ctl, S.G, S.F);
            else if (lane == 0) carry_slot(ci, S.clk[slot_out], S.clk[slot_nx]);
            __syncwarp();
            if (lane == 0) write_status(S.clk[slot_out], S.status);
        }
        __syncwarp();
    }
}

}  // namespace sw2d
