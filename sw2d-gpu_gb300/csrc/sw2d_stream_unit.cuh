// sw2d_stream_unit.cuh -- one warp's work in the FP32 streaming scheme: a
// strip of rows of a 32-column window of one scenario (27 output columns).
//
// Shared by the single-scenario streaming kernel (sw2d_stream.cuh) and the
// batched kernel (sw2d_batch.cuh); the arithmetic is that of step_kernel in
// sw2d_device.cuh, organised as a 3-row register pipeline (see
// sw2d_stream.cuh for the layout of the pipeline and the halo).
#pragma once

#include <cuda.h>

#include "sw2d_device.cuh"

namespace sw2d {

// ---- rows staged in shared memory by TMA (the stream_step_tma_kernel build) ----
//
// Tensor maps of the planes a launch reads (pitched layout, frame included);
// the copies address cells by plane coordinates (column + 4, row + 4).
struct TmaMaps {
    CUtensorMap h[2], um[2], vn[2], r[2], dzx, dzy, n, m;
};
constexpr int kTmaStages = 4;                 // row stages per warp
constexpr int kTmaSlot = 256;                 // bytes per field box in a stage (128-byte aligned)
constexpr int kTmaStageBytes = 8 * kTmaSlot;  // h, um, vn, n, remainder, dzx, dzy, mask
constexpr int kTmaBoxF = 40;                  // FP32 box width: the window, its neighbours, alignment slack
constexpr int kTmaBoxM = 48;                  // mask box width in bytes

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_inval(unsigned long long *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Waits for the phase of parity `ph` with a bounded number of polls; false
// when it gave up (the caller reports an error instead of hanging).
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned ph) {
    for (int it = 0; it < (1 << 22); it++) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(ph)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// One row box of a plane into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_row(unsigned dst, const CUtensorMap *map, int x, int y, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"((unsigned long long)map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Halo lanes: lanes whose results are incomplete because a neighbour they
// need lies outside the window (the shuffles return a lane's own value at the
// window's edges).  West: each lane loads its west neighbour's depth instead
// of shuffling it, so the face velocities of lane 0 are exact; its discharges
// are not (they need lane -1's velocities), lane 1's are; so the dry-cell
// flags are exact from lane 1, the final depths from lane 2 (the west face
// tests the west cell's flag) and the CFL bounds of the y-faces, which take
// the west cell's final depth, from lane 3.  East: each lane loads its east
// neighbour's depth and y discharge and computes that lane's y-face velocity
// itself, so the y discharges of lane 31 are exact too; its x discharges are
// not (the corner flux east of it is its east neighbour's, taken by a
// shuffle) and neither is its provisional depth (it needs lane 32's y-face
// discharge), so the dry-cell flags are exact up to lane 30 and the final
// depths up to lane 29 (the east face tests the east cell's flag).  Loading
// a neighbour's values in place of a shuffle costs the same issue slot;
// recomputing lane -1's velocities as well (a 2-lane west halo) cost more
// than the lane saved.
constexpr int kStreamHL = 3;                            // west halo lanes
constexpr int kStreamHR = 2;                            // east halo lanes
constexpr int kStreamOut = 32 - kStreamHL - kStreamHR;  // output columns per warp
constexpr int kStreamMaxSrc = 16;                       // point sources per warp strip

__device__ __forceinline__ float shup(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ float shdn(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }

// Upwinded flux through one side of a control volume.  The reference writes
// it as vel*(o+s)/2 + |vel|*(s-o)/2 (cu:174, and its mirror cu:175) with vel
// an average of two face velocities; that equals vel * (vel >= 0 ? s : o),
// which the FP32 path evaluates with one select.  Here `vel2` is the sum of
// the two face velocities: the halves are folded into dt2/dx and dt2/dy.
__device__ __forceinline__ float upw(float vel2, float o, float s) { return vel2 * (vel2 >= 0.f ? s : o); }
__device__ __forceinline__ float upw_r(float vel2, float o, float s) { return vel2 * (vel2 >= 0.f ? o : s); }

// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker's fast two-sum,
// written without contraction or reassociation).
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// Dry-bed rules (cu:130-159 / cu:247-276) of a face between cells a (north /
// west) and b, with the bed entering only as dz = z_b - z_a: the reference's
// hb + zb < za is hb + dz < 0, ha + za < zb is ha < dz, and its
// max(eta) - max(z) is max(hb + dz, ha) - max(dz, 0) (all shifted by z_a).
// Returns true and sets q when a rule applies.
__device__ __forceinline__ bool dry_bed_dz(const Thr<float> &T, float g, float ha, float hb, float dz, float &q) {
    if (hb + dz < 0.f) {  // cu:130
        q = (ha >= T.gt_th) ? 0.5440f * ha * sqrtf(g * ha) : 0.f;
        return true;
    }
    if (ha < dz) {  // cu:138
        q = (hb >= T.gt_th) ? -0.544f * hb * sqrtf(g * hb) : 0.f;
        return true;
    }
    // cu:149: exactly one side strictly wet, with comparisons false for NaN
    const bool b_wet = hb >= T.gt_th, a_wet = ha >= T.gt_th;
    const bool b_dry = hb < T.ge_th, a_dry = ha < T.ge_th;
    if ((b_wet && a_dry) || (b_dry && a_wet)) {
        if ((hb > 0.f) || (ha > 0.f)) {
            const float s = b_wet ? -0.350f : 0.350f;  // cu:151-154
            const float hh3 = fmaxf(hb + dz, ha) - fmaxf(dz, 0.f);
            q = s * hh3 * sqrtf(2.00f * g * hh3);
        } else {
            q = 0.f;
        }
        return true;
    }
    return false;
}

// Everything a warp reads to advance one strip of one scenario.
struct StreamView {
    int rows, cols, pitch, south_open;
    const float *Hin, *Uin, *Vin, *Nin;  // Nin == nullptr: scalar Manning n
    const float *DZX, *DZY;              // bed differences across x- / y-faces (pack_dz_kernel)
    const float *Rin;                    // depth remainders of the state read (compensated depth)
    float *Rout;                         // and of the state written
    const uint8_t *Min;
    const float *Win;  // per-cell rain factors or nullptr (uniform rain)
    float *Hout, *Uout, *Vout;
    GridScalars<float> GS;
    Thr<float> T;
    LaunchScalars<float> LS;
    bool storm, on0, on1;
    int n_src;                 // point sources of the scenario
    const ForcingDesc *F;      // tables of the sources (only read when n_src > 0)
    double t0, t1, dx, dy;     // for the source rates (FP64, once per warp)
};

// Lane 0's copy of a value, for the whole warp: a value the compiler can see
// to be warp-uniform lives in a uniform register instead of one per thread.
__device__ __forceinline__ int wuni(int v) { return __shfl_sync(0xffffffffu, v, 0); }
__device__ __forceinline__ float wuni(float v) { return __shfl_sync(0xffffffffu, v, 0); }
template <class T>
__device__ __forceinline__ T *wuni(T *p) {
    return reinterpret_cast<T *>(__shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(p), 0));
}

// Per-warp results of a strip (per lane until reduced).
struct StreamAcc {
    float rain, src, ev, out, clamp, cm;
    bool bad;
    bool too_many_sources;
};

// Advances column tile `ct`, rows r0 .. r1-1 (a strip) of the
// scenario in V.  s_sr/s_sc/s_q0/s_q1 are this warp's slots for local point
// sources (kStreamMaxSrc each).  UNR is the unrolling of the row loop;
// RAINW builds in the per-cell rain factors (V.Win) and GEN the moving storm
// and the point sources; the builds without them leave that code out
// entirely, because even unexecuted it slowed the row loop (the rain factors
// by 6-11 %, the storm and sources by 9 %, as instructions fetched past and
// registers held, not as work).
//
// Domain edges need no tests of their own: the zero frame around every field
// has mask 0, so the face tests on the two cells' masks already close the
// walls and skip everything outside the domain; wall discharges are 0, so
// the face velocities there are 0 whatever face depth divides them; and the
// frame row below the last cell row holds a copy of that row's depth, so the
// plain average 0.5*(x + x) = x is the reference's face depth at the south
// face (cu:380-381), used by the open south edge.  Two rules of the
// reference stay explicit: no cross advection u12 on column 0 (cu:178-180)
// and no v11 on row 0 (cu:289-291).
//
// TMA: the rows come from shared memory, copied there by TMA (maps M, buffer
// parity buf, the warp's kTmaStages stages at stg and their barriers at
// bars) instead of being loaded by every lane.
//
// PIPE: the state is read past the L1 cache (ld.global.cg): in the pipelined
// launches other SMs rewrite the state between this warp's iterations, so a
// line this SM cached in an earlier iteration must not be read again.  Once
// the strip's first three output rows are written (all that the strip
// above reads of this iteration) and the rows above the strip have been
// read (all of the strip above that this iteration reads), lane 0 publishes
// top_val at *top_flag with a release store.
template <int UNR, bool RAINW, bool GEN, bool TMA = false, bool PIPE = false>
__device__ __forceinline__ void stream_unit(const StreamView &V, const int ct, const int r0, const int r1,
                                            const int lane, int *s_sr, int *s_sc, float *s_q0, float *s_q1,
                                            StreamAcc &A, const TmaMaps *M = nullptr, int buf = 0,
                                            unsigned char *stg = nullptr, unsigned long long *bars = nullptr,
                                            unsigned *top_flag = nullptr, unsigned top_val = 0u) {
    const int rows = wuni(V.rows), cols = wuni(V.cols), pitch = wuni(V.pitch), south_open = wuni(V.south_open);
    const float dt2 = wuni(V.LS.dt2), dt2dx = wuni(V.LS.dt2dx), dt2dy = wuni(V.LS.dt2dy);
    const float u_ev0 = wuni(V.LS.ev0), u_ev1 = wuni(V.LS.ev1), u_rr0 = wuni(V.LS.rr0), u_rr1 = wuni(V.LS.rr1);
    const float sx0 = wuni(V.LS.sx0), sy0 = wuni(V.LS.sy0), sx1 = wuni(V.LS.sx1), sy1 = wuni(V.LS.sy1);
    const float storm_amp = wuni(V.GS.storm_amp), storm_2s2 = wuni(V.GS.storm_2s2);
    const int storm = GEN ? wuni((int)V.storm) : 0, on0 = wuni((int)V.on0), on1 = wuni((int)V.on1);
    const float hdx = 0.5f * dt2dx, hdy = 0.5f * dt2dy;  // dt2/dx, dt2/dy times the halves of upw()
    const float hdt2 = 0.5f * dt2;  // the dt2 * ram / 2 of cu:203 and cu:320, as hdt2 * ram
    const float dx = wuni(V.GS.dx), dy = wuni(V.GS.dy), g = wuni(V.GS.g), manning = wuni(V.GS.manning);
    const float rdx = wuni(V.GS.rdx), rdy = wuni(V.GS.rdy);
    const float pct_hi = wuni(V.GS.pct_hi), pct_lo = wuni(V.GS.pct_lo);
    const float gt_th = wuni(V.T.gt_th), ge_th = wuni(V.T.ge_th), gt_ev = wuni(V.T.gt_evmin);
    Thr<float> T;
    T.gt_th = gt_th;
    T.ge_th = ge_th;
    T.gt_evmin = gt_ev;
    // continuity (cu:603-665) in the uniform-rain form (no storm, sources or
    // rain factors): -dt2/dx, -dt2/dy, and the forcing dt2 (rr pct - ev) by
    // whether the old depth is above EV_WL_min, at t (f0) and t + dt (f1)
    const float ndx = -dt2 * rdx, ndy = -dt2 * rdy;
    const float f0_hi = dt2 * (u_rr0 * pct_hi - u_ev0), f0_lo = dt2 * (u_rr0 * pct_lo);
    const float f1_hi = dt2 * (u_rr1 * pct_hi - u_ev1), f1_lo = dt2 * (u_rr1 * pct_lo);
    const float sqrt_g = sqrtf(g);
    // |q/h| + sqrt(g h) with one reciprocal square root: r = 1/sqrt(h)
    auto wave_speed = [&](float q, float h) {
        const float r = rsqrtf(h);
        return fabsf(q) * r * r + sqrt_g * h * r;
    };
    // Manning friction coefficient g n^2 |u| / h^(4/3) (cu:194-199, cu:311-316),
    // with n the mean of the two cells' n (given as their sum sn) and h^(-4/3) as
    // 2^(-1.3333330 log2 h); zero when h <= th or n == 0
    // g (n_a + n_b)^2 / 4 = g n_face^2, and g dt2/dx, g dt2/dy of the surface-slope
    // terms (cu:166, cu:283), formed once per warp instead of per face
    const float g4 = 0.25f * g;
    const float gdx = g * dt2dx, gdy = g * dt2dy;
    auto friction = [&](float sn, float speed2, float h) {  // sn = n_a + n_b
        const float ram = g4 * sn * sn * sqrtf(speed2) * exp2f(-1.3333330f * __log2f(h));
        return (!(h < gt_th) && sn != 0.f) ? ram : 0.f;
    };
    const bool raster = V.Nin != nullptr;
    const float *__restrict__ Hin = wuni(V.Hin);
    const float *__restrict__ Uin = wuni(V.Uin);
    const float *__restrict__ Vin = wuni(V.Vin);
    const float *__restrict__ DZX = wuni(V.DZX);
    const float *__restrict__ DZY = wuni(V.DZY);
    const float *__restrict__ Rin = wuni(V.Rin);
    float *__restrict__ Rout = wuni(V.Rout);
    const float *__restrict__ Nin = wuni(V.Nin);
    const uint8_t *__restrict__ Min = wuni(V.Min);
    const float *__restrict__ Win = wuni(V.Win);
    float *__restrict__ Hout = wuni(V.Hout);
    float *__restrict__ Uout = wuni(V.Uout);
    float *__restrict__ Vout = wuni(V.Vout);

    const int gj0 = ct * kStreamOut - kStreamHL;
    const int gj = gj0 + lane;
    const int R0 = r0, R1 = r1;
    const bool out_col = lane >= kStreamHL && lane < kStreamHL + kStreamOut && gj < cols;
    const bool not_col0 = gj != 0;

    // point sources inside this warp's window, in list order (the later one
    // wins on a shared cell, as the reference's assignment, cu:545)
    int nsrc = 0;
    if (GEN && V.n_src > 0) {
        const double area = V.dx * V.dy;
        for (int base = 0; base < V.n_src; base += 32) {
            const int s = base + lane;
            bool in = false;
            int sr = 0, sc = 0;
            if (s < V.n_src) {
                const int cell = V.F->src_cell[s];
                sr = cell / cols;
                sc = cell - sr * cols;
                in = sr >= R0 - 4 && sr < R1 + 3 && sc >= gj0 && sc < gj0 + 32;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            if (in) {
                const int off = nsrc + __popc(bal & ((1u << lane) - 1u));
                if (off < kStreamMaxSrc) {
                    s_sr[off] = sr;
                    s_sc[off] = sc;
                    s_q0[off] = (float)source_rate(*V.F, V.n_src, s, V.t0, area);
                    s_q1[off] = (float)source_rate(*V.F, V.n_src, s, V.t1, area);
                } else {
                    A.too_many_sources = true;
                }
            }
            nsrc += __popc(bal);
        }
        __syncwarp();
        nsrc = min(nsrc, kStreamMaxSrc);
    }
    auto source_at = [&](int row, bool second) -> float {
        float q = 0.f;
        for (int e = 0; e < nsrc; e++)
            if (s_sr[e] == row && s_sc[e] == gj) q = second ? s_q1[e] : s_q0[e];
        return q;
    };
    auto storm_rate = [&](int row, bool on, float sx, float sy) -> float {
        if (!on) return 0.f;
        const float x = ((float)gj + 0.5f) * dx - sx;
        const float y = ((float)row + 0.5f) * dy - sy;
        return storm_amp * __expf(-(x * x + y * y) / storm_2s2);
    };

    // row loads: rows R0-4 .. R1+2 (the bed differences R0-4 .. R1+1) and
    // columns gj0-1 .. gj0+32 (the window and
    // the neighbours loaded at its edges; gj0 >= -3, and the last window ends
    // 29 columns past the east wall) all lie inside the zero frame around the
    // domain, whose zeros are the inactive-cell and wall values, so no load
    // needs a bounds test
    float p_h, p_hw, p_hE, p_vnE, p_dzx, p_dzy, p_n, p_um, p_vn, p_res;
    unsigned p_m;
    int gp = (R0 - 4) * pitch + gj;  // element offset of the next row to read (fields fit 32-bit offsets)
    const int gp0 = gp;
    int lrow = R0 - 4;  // row of the next load
    auto ld_state = [](const float *p) -> float {
        if constexpr (PIPE) return __ldcg(p);
        else return *p;
    };
    auto load_row_global = [&]() {
        p_h = ld_state(Hin + gp);
        p_hw = ld_state(Hin + gp - 1);  // the west neighbour's depth, exact on lane 0 too
        p_res = lrow >= 3 ? ld_state(Rin + gp - 3 * pitch) : 0.f;  // remainder of row lrow-3, used with this row
        lrow++;
        p_n = raster ? Nin[gp] : manning;
        p_m = (unsigned)Min[gp];
        p_um = ld_state(Uin + gp);
        p_vn = ld_state(Vin + gp);
        p_hE = ld_state(Hin + gp + 1);  // the east neighbour's depth and discharges
        p_vnE = ld_state(Vin + gp + 1);
        gp += pitch;
    };

    const int r_first = R0 - 4, r_last = R1 + 3;
    // TMA build: each warp keeps rows in kTmaStages stages, copied
    // kTmaStages - 1 rows ahead of the row read from them; the stage of row k
    // holds h, um, vn, n and the mask of row k, the remainder of row k - 3 and
    // the bed differences of row k - 1.  Box origins are rounded down to a
    // 16-byte boundary (4 FP32 columns, 16 mask bytes); the plane coordinates
    // (column + 4, row + 4) are >= 0 except the remainder rows above the
    // frame, which the copy fills with zeros (as the register build's 0).
    // Every operand of a copy is warp-uniform (broadcast from lane 0).
    const int xf = TMA ? wuni((gj0 + 3) & ~3) : 0, xm = TMA ? wuni((gj0 + 4) & ~15) : 0;
    const int of = gj + 4 - xf, om = gj + 4 - xm;  // this lane's index in the boxes
    const unsigned stg_s = TMA ? (unsigned)wuni((int)smem_u32(stg)) : 0u;
    const unsigned bars_s = TMA ? (unsigned)wuni((int)smem_u32(bars)) : 0u;
    const int ub = TMA ? wuni(buf) : 0;
    const unsigned tx = (unsigned)((raster ? 7 : 6) * kTmaBoxF * 4 + kTmaBoxM);
    auto issue = [&](int k) {  // one lane: row k into its stage
        const int s = (k - r_first) % kTmaStages;
        const unsigned st = stg_s + s * kTmaStageBytes, bar = bars_s + s * 8;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(tx) : "memory");
        const int y = k + 4;
        tma_row(st + 0 * kTmaSlot, &M->h[ub], xf, y, bar);
        tma_row(st + 1 * kTmaSlot, &M->um[ub], xf, y, bar);
        tma_row(st + 2 * kTmaSlot, &M->vn[ub], xf, y, bar);
        if (raster) tma_row(st + 3 * kTmaSlot, &M->n, xf, y, bar);
        tma_row(st + 4 * kTmaSlot, &M->r[ub], xf, y - 3, bar);
        tma_row(st + 5 * kTmaSlot, &M->dzx, xf, y - 1, bar);
        tma_row(st + 6 * kTmaSlot, &M->dzy, xf, y - 1, bar);
        tma_row(st + 7 * kTmaSlot, &M->m, xm, y, bar);
    };
    auto load_row_tma = [&]() {
        const int k = lrow - r_first;
        const unsigned char *st = stg + (k % kTmaStages) * kTmaStageBytes;
        if (!mbar_wait(bars_s + (k % kTmaStages) * 8, (unsigned)((k / kTmaStages) & 1))) A.bad = true;
        const float *fh = reinterpret_cast<const float *>(st);
        p_h = fh[of];
        p_hw = fh[of - 1];
        p_hE = fh[of + 1];
        p_um = reinterpret_cast<const float *>(st + kTmaSlot)[of];
        const float *fv = reinterpret_cast<const float *>(st + 2 * kTmaSlot);
        p_vn = fv[of];
        p_vnE = fv[of + 1];
        p_n = raster ? reinterpret_cast<const float *>(st + 3 * kTmaSlot)[of] : manning;
        p_res = reinterpret_cast<const float *>(st + 4 * kTmaSlot)[of];
        p_dzx = reinterpret_cast<const float *>(st + 5 * kTmaSlot)[of];
        p_dzy = reinterpret_cast<const float *>(st + 6 * kTmaSlot)[of];
        p_m = (unsigned)(st + 7 * kTmaSlot)[om];
        lrow++;
        // the stage read before this one is free once every lane is past it;
        // the proxy fence orders those reads before the copy that refills it
        __syncwarp();
        if (lrow - 1 + kTmaStages - 1 < r_last && lane == 0) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(lrow - 1 + kTmaStages - 1);
        }
    };
    auto load_row = [&]() {
        if constexpr (TMA) load_row_tma();
        else load_row_global();
    };

    // register rings: suffix = rows back from the row being read (r)
    float h1 = 0.f, h2 = 0.f, h3 = 0.f, hL1 = 0.f;
    float n1 = manning, n2 = manning, nL1 = manning;
    float um1 = 0.f, um2 = 0.f, vn1 = 0.f, vn2 = 0.f;
    float uu_1 = 0.f, uu_2 = 0.f, uuL_1 = 0.f;
    float vv_1 = 0.f, vv_2 = 0.f, vvR_1 = 0.f, vvR_2 = 0.f;
    float vnE1 = 0.f;  // the east neighbour's y discharge of row r-1
    float rum_2 = 0.f, rum_3 = 0.f, rvn_2 = 0.f, rvn_3 = 0.f;
    float hw_4 = 0.f;
    float fx_1 = 0.f, cy_1 = 0.f;    // x flux through the cell north of the face, corner y flux (previous row)
    float hmf_1 = 0.f, hnf_1 = 0.f;  // face depths of row r-1
    unsigned mb = 0u, mLb = 0u;  // bit k: active mask of row r-k (own / west column)
    unsigned db = 0u;            // bit k: row r-2-k is active and dry after the provisional update

    if constexpr (TMA) {
        if (lane == 0)
            for (int k = r_first; k < r_first + kTmaStages - 1 && k < r_last; k++) issue(k);
    }
    load_row();
    if constexpr (!TMA) {
        p_dzx = 0.f;  // the bed differences of row r_first - 1 are not used
        p_dzy = 0.f;
    }
#pragma unroll UNR
    for (int r = r_first; r < r_last; r++) {
        const float hE0 = p_hE, vnE0 = p_vnE;
        const float h0 = p_h, hL0 = p_hw, n0 = p_n, um0 = p_um, vn0 = p_vn;
        const float res3 = p_res;  // depth remainder of row r-3
        mb = (mb << 1) | p_m;
        const unsigned mL0 = __shfl_up_sync(0xffffffffu, p_m, 1);
        mLb = (mLb << 1) | mL0;
        float dzx1 = p_dzx, dzy1 = p_dzy;  // bed differences of row r-1
        if constexpr (TMA) {  // row r's stage holds those of row r-1; row r_first - 1's are not used
            dzx1 = r > r_first ? dzx1 : 0.f;
            dzy1 = r > r_first ? dzy1 : 0.f;
        }
        if (r + 1 < r_last) load_row();  // prefetch the next row
        if constexpr (!TMA) {
            // the bed differences are used one row after they are read, so
            // they are read one row late (row r, for the next iteration)
            // instead of passing through a register ring
            p_dzx = DZX[(r - r_first) * pitch + gp0];
            p_dzy = DZY[(r - r_first) * pitch + gp0];
        }

        const float nL0 = raster ? shup(n0) : manning;
        // ---- row r: face velocities (cu:363-453) ----
        const float hnf = 0.50f * (h0 + hL0);
        const float vv_0 = (hnf >= ge_th) ? vn0 / hnf : 0.0f;
        const float hmf = 0.50f * (h0 + h1);
        const float uu_0 = (hmf >= ge_th) ? um0 / hmf : 0.0f;
        const float uuL_0 = shup(uu_0);
        // the east neighbour's y-face velocity, as that lane computes it
        const float hnfE = 0.50f * (hE0 + h0);
        const float vvE_0 = (hnfE >= ge_th) ? vnE0 / hnfE : 0.0f;

        // ---- row r-1: new face discharges (cu:98-354) ----
        const int i = r - 1;
        const float umW = shup(um1);
        const float vnE = vnE1;
        // upwinded fluxes shared between neighbouring faces: the flux through
        // the cell south of x-face i is the one north of face i+1 (kept for the
        // next row); the corner flux east of a lane is the one west of its east
        // neighbour (a shuffle); likewise along the rows for the y-faces
        const float vx = uu_0 + uu_1;
        const float fx_0 = vx * (vx >= 0.f ? um1 : um0);  // upw(uu_0 + uu_1, um0, um1)
        const float vw2 = vv_1 + vv_2;
        const float fw = vw2 * (vw2 >= 0.f ? umW : um1);  // upw_r(vv_1 + vv_2, umW, um1)
        const float fe = shdn(fw);                        // the east lane's fw (lane 31: a halo lane)
        const float vc = uu_0 + uuL_0;
        const float cy_0 = vc * (vc >= 0.f ? vn1 : vn0);  // upw(uu_0 + uuL_0, vn0, vn1)
        const float ve2 = vvR_1 + vv_1;
        const float ge = ve2 * (ve2 >= 0.f ? vn1 : vnE);  // upw(vvR_1 + vv_1, vnE, vn1)
        const float gw = shup(ge);                        // the west lane's ge (lane 0: a halo lane)
        float rum_1 = 0.f;
        {
            const float ha = h2, hb = h1, dz = dzx1;
            if (((mb >> 2) & (mb >> 1) & 1u) && ((ha >= gt_th) || (hb >= gt_th))) {
                if (!dry_bed_dz(T, g, ha, hb, dz, rum_1)) {
                    const float hm = hmf_1;  // 0.5 (hb + ha), formed with the velocities
                    const float u13 = gdx * hm * ((hb - ha) + dz);  // cu:166, hb + zb - ha - za
                    const float u11 = hdx * (fx_0 - fx_1);
                    const float u12c = hdy * (fe - fw);
                    const float u12 = not_col0 ? u12c : 0.f;  // zero on column 0 (cu:178-180)
                    const float vva = 0.250f * (vv_1 + vvR_1 + vv_2 + vvR_2);
                    const float ram = friction(n1 + n2, uu_1 * uu_1 + vva * vva, hm);
                    const float x = hdt2 * ram;
                    rum_1 = ((1.00f - x) * um1 + (-u11 - u12 - u13)) / (1.00f + x);  // cu:203
                }
            } else if (i == rows && south_open) {  // free outfall (extension)
                if (((mb >> 2) & 1u) && h2 >= gt_th) rum_1 = 0.5440f * h2 * sqrtf(g * h2);
            }
        }
        float rvn_1 = 0.f;
        {
            const float ha = hL1, hb = h1, dz = dzy1;
            if (((mLb >> 1) & (mb >> 1) & 1u) && ((ha >= gt_th) || (hb >= gt_th))) {
                if (!dry_bed_dz(T, g, ha, hb, dz, rvn_1)) {
                    const float hn = hnf_1;
                    const float v13 = gdy * hn * ((hb - ha) + dz);  // cu:283, hb + zb - ha - za
                    const float v11c = hdx * (cy_0 - cy_1);
                    const float v11 = (i != 0) ? v11c : 0.f;  // zero on row 0 (cu:289-291)
                    const float v12 = hdy * (ge - gw);
                    const float uua = 0.250f * (uu_1 + uu_0 + uuL_1 + uuL_0);
                    const float ram = friction(n1 + nL1, uua * uua + vv_1 * vv_1, hn);
                    const float x = hdt2 * ram;
                    rvn_1 = ((1.00f - x) * vn1 + (-v11 - v12 - v13)) / (1.00f + x);  // cu:320
                }
            }
        }

        // ---- row r-2: provisional depth, forcing at t (cu:1278-1288) ----
        const float rvnE_2 = shdn(rvn_2);
        float hs_2 = 0.f;
        if ((mb >> 2) & 1u) {
            const float ho = h2;
            const bool hi = ho >= gt_ev;
            const float pct = hi ? pct_hi : pct_lo;
            const float evapo = hi ? u_ev0 : 0.f;
            const float ql = nsrc ? source_at(r - 2, false) : 0.f;
            float rr = storm ? storm_rate(r - 2, on0, sx0, sy0) : u_rr0;
            if (RAINW) rr = rr * Win[(r - 2) * pitch + gj];
            if constexpr (!GEN && !RAINW) {  // the cell's forcing is one select of per-warp values
                hs_2 = fmaxf(ho + ((rum_1 - rum_2) * ndx + (rvnE_2 - rvn_2) * ndy) + (hi ? f0_hi : f0_lo), 0.f);
            } else {
                hs_2 = fmaxf(ho - dt2 * ((rum_1 - rum_2) * rdx + (rvnE_2 - rvn_2) * rdy - ql - rr * pct + evapo),
                             0.f);
            }
        }

        // ---- row r-3: dry-cell fix (cu:695-725) and final depth ----
        // dry-cell fix (cu:695-725): a cell is "dry" when active and h* < th; its
        // flag is kept in a bit ring, so each cell's test is made once
        db = (db << 1) | ((((mb >> 2) & 1u) && hs_2 < ge_th) ? 1u : 0u);
        const unsigned dbW = __shfl_up_sync(0xffffffffu, db, 1);
        const bool m3 = (mb >> 3) & 1u, m4 = (mb >> 4) & 1u, mL3 = (mLb >> 3) & 1u;
        const bool d2 = db & 1u, d3 = (db >> 1) & 1u, d4 = (db >> 2) & 1u, dW3 = (dbW >> 1) & 1u;
        float un = rum_3;  // x-face north of the row-(r-3) cell
        if ((un > 0.f && d4) || (un < 0.f && d3)) un = 0.f;
        float us = rum_2;  // x-face south of it
        if ((us > 0.f && d3) || (us < 0.f && d2)) us = 0.f;
        float vw = rvn_3;  // y-face west of it
        if ((vw > 0.f && dW3) || (vw < 0.f && d3)) vw = 0.f;
        const float ve = shdn(vw);
        const int f = r - 3;
        float hw_3 = 0.f, hres = 0.f, clampv = 0.f, rr1 = 0.f, pct1 = 0.f, ev1 = 0.f, ql1 = 0.f;
        if (m3) {
            const float ho = h3;
            const bool hi = ho >= gt_ev;
            pct1 = hi ? pct_hi : pct_lo;
            ev1 = hi ? u_ev1 : 0.f;
            ql1 = nsrc ? source_at(f, true) : 0.f;
            rr1 = storm ? storm_rate(f, on1, sx1, sy1) : u_rr1;
            if (RAINW) rr1 = rr1 * Win[f * pitch + gj];
            // compensated depth: the state is the FP32 pair h + remainder, and the
            // update is added with two error-free sums, so that changes below half
            // an ulp of h (light rain on deep water) accumulate in the remainder
            // instead of being rounded away, which would leave the FP32 state
            // behind its FP64 budget.  The fast two-sum is exact here: an update
            // larger than the depth either drains the cell (clamped below) or
            // fills it from 0, and the remainder is below an ulp of the depth.
            float d;
            if constexpr (!GEN && !RAINW) {
                d = (us - un) * ndx + (ve - vw) * ndy + (hi ? f1_hi : f1_lo);
            } else {
                d = __fmul_rn(-dt2, (us - un) * rdx + (ve - vw) * rdy - ql1 - rr1 * pct1 + ev1);
            }
            float s, e, hn, rn;
            fast_two_sum(ho, d, s, e);
            fast_two_sum(s, __fadd_rn(res3, e), hn, rn);
            if (hn < 0.f) {  // fmax(h, 0) (cu:657) of the pair
                clampv = -__fadd_rn(hn, rn);
                hn = 0.f;
                rn = 0.f;
            }
            hw_3 = hn;
            hres = rn;
        }
        const float hwW = shup(hw_3);
        if (out_col && f >= R0) {  // f <= R1 - 1 always
            const int gp = f * pitch + gj;
            Hout[gp] = hw_3;
            Rout[gp] = hres;
            Uout[gp] = un;
            Vout[gp] = vw;
            if (f == rows - 1) {  // south face, and the depth copy below the last row
                Uout[gp + pitch] = us;
                Hout[gp + pitch] = hw_3;
                A.out += us;
            }
            if (m3) {
                A.rain += rr1 * pct1;
                A.src += ql1;
                A.ev += ev1;
                A.clamp += clampv;
                // CFL bound of the new state on the owned faces (extension)
                if (m4) {
                    const float hm = 0.50f * (hw_3 + hw_4);
                    if (hm >= ge_th) A.cm = fmaxf(A.cm, wave_speed(un, hm));
                }
                if (f == rows - 1 && south_open && hw_3 >= ge_th)
                    A.cm = fmaxf(A.cm, wave_speed(us, hw_3));
                if (mL3) {
                    const float hn = 0.50f * (hw_3 + hwW);
                    if (hn >= ge_th) A.cm = fmaxf(A.cm, wave_speed(vw, hn));
                }
            }
            if (!isfinite(hw_3 + un + vw)) A.bad = true;  // a NaN or an infinity in any of the three
        }

        if constexpr (PIPE) {
            if (r == R0 + 5) {  // output rows R0 .. R0+2 written; every row above R0 read
                __syncwarp();
                if (lane == 0)
                    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(top_flag), "r"(top_val) : "memory");
            }
        }

        // ---- advance the rings ----
        h3 = h2; h2 = h1; h1 = h0; hL1 = hL0;
        n2 = n1; n1 = n0; nL1 = nL0;
        um2 = um1; um1 = um0; vn2 = vn1; vn1 = vn0;
        uu_2 = uu_1; uu_1 = uu_0; uuL_1 = uuL_0;
        vv_2 = vv_1; vv_1 = vv_0; vvR_2 = vvR_1; vvR_1 = vvE_0;
        vnE1 = vnE0;
        rum_3 = rum_2; rum_2 = rum_1; rvn_3 = rvn_2; rvn_2 = rvn_1;
        hw_4 = hw_3;
        fx_1 = fx_0; cy_1 = cy_0;
        hmf_1 = hmf; hnf_1 = hnf;
    }
}

// Warp reduction of a StreamAcc: sums / max / any into lane 0's return.
__device__ __forceinline__ void warp_reduce_acc(StreamAcc &A) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        A.rain += __shfl_xor_sync(0xffffffffu, A.rain, o);
        A.src += __shfl_xor_sync(0xffffffffu, A.src, o);
        A.ev += __shfl_xor_sync(0xffffffffu, A.ev, o);
        A.out += __shfl_xor_sync(0xffffffffu, A.out, o);
        A.clamp += __shfl_xor_sync(0xffffffffu, A.clamp, o);
        A.cm = fmaxf(A.cm, __shfl_xor_sync(0xffffffffu, A.cm, o));
    }
    A.bad = __any_sync(0xffffffffu, A.bad);
    A.too_many_sources = __any_sync(0xffffffffu, A.too_many_sources);
}

}  // namespace sw2d
