// sw2d_stream.cuh -- FP32 warp-streaming step kernel.
//
// The same iteration as step_kernel (one iteration of the reference loop
// SW2D-GPU_linux/src/SW2D-GPU.cu:1256-1336, "cu:<line>" below), organised
// for the FP32 path's instruction budget instead of for FP64 reuse:
//
//   * one warp owns 32 adjacent columns -- 25 output columns plus 4 halo
//     columns on the west and 3 on the east, the lateral dependency radius
//     of one iteration (+1 for the CFL ring) -- and marches down a strip of
//     rows;
//   * each row read from HBM (h, z, n, mask, um, vn; one coalesced 128-byte
//     line per field and warp) feeds a 3-row register pipeline
//         row r    : face depths and velocities uu1/vv1        (cu:363-453)
//         row r-1  : new face discharges, momentum + dry bed   (cu:98-354)
//         row r-2  : provisional depth, forcing at t           (cu:603-665)
//         row r-3  : dry-cell fix per face (cu:695-725), final depth with
//                    forcing at t+dt, CFL bound of the owned faces
//     so every quantity is computed once per cell and row, in registers;
//   * west/east neighbours come from warp shuffles; there is no shared-memory
//     tile and no block-wide barrier inside the row loop;
//   * the next row's loads are issued before the current row's arithmetic.
//
// Budgets and the CFL bound are reduced per warp and then per CTA; the last
// CTA of the launch finalises the clock slot (finish_cta).
#pragma once

#include "sw2d_device.cuh"

namespace sw2d {

constexpr int kStreamHL = 4;                            // west halo lanes (3 + CFL ring)
constexpr int kStreamHR = 3;                            // east halo lanes
constexpr int kStreamOut = 32 - kStreamHL - kStreamHR;  // output columns per warp
constexpr int kStreamMaxSrc = 16;                       // point sources per warp strip

struct StreamShape {
    int tiles_w;  // column tiles of kStreamOut columns
    int strip_h;  // output rows per warp
    int units;    // tiles_w * number of strips
    int pad;
};

__device__ __forceinline__ float shup(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ float shdn(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }

template <int NWARP, int MINB, int UNROLL>
__global__ void __launch_bounds__(NWARP * 32, MINB)
    stream_step_kernel(const GridDesc G, const ForcingDesc F, const StateBufs<float> S, const Thr<float> T,
                       Clock *__restrict__ clk, const Control *__restrict__ ctl, const int slot,
                       const StreamShape SH) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int slot_out = slot == 2 ? 0 : slot + 1;
    const int slot_nx = slot == 0 ? 2 : slot - 1;
    const Clock &ci = clk[slot];
    if (!ci.plan.run) {
        if (blockIdx.x == 0 && tid == 0) carry_slot(ci, clk[slot_out], clk[slot_nx]);
        return;
    }

    __shared__ int s_sr[NWARP][kStreamMaxSrc], s_sc[NWARP][kStreamMaxSrc];
    __shared__ float s_q0[NWARP][kStreamMaxSrc], s_q1[NWARP][kStreamMaxSrc];
    __shared__ float s_red[NWARP][B_N + 1];
    __shared__ int s_bad[NWARP];

    const LaunchScalars<float> LS = ci.plan.f;
    const GridScalars<float> &GS = G.sf;
    const int rows = G.rows, cols = G.cols, pitch = G.pitch;
    const float dt2 = LS.dt2, dt2dx = LS.dt2dx, dt2dy = LS.dt2dy;
    const float dx = GS.dx, dy = GS.dy, g = GS.g, manning = GS.manning, rdx = GS.rdx, rdy = GS.rdy;
    const float pct_hi = GS.pct_hi, pct_lo = GS.pct_lo;
    const float gt_th = T.gt_th, ge_th = T.ge_th, gt_ev = T.gt_evmin;
    const bool raster = S.nman != nullptr;
    const bool storm = F.rain_kind == RAIN_STORM;
    const bool on0 = ci.plan.storm_on0, on1 = ci.plan.storm_on1;
    const int buf = ci.buf;
    const float *__restrict__ Hin = S.h[buf];
    const float *__restrict__ Uin = S.um[buf];
    const float *__restrict__ Vin = S.vn[buf];
    const float *__restrict__ Zin = S.z;
    const float *__restrict__ Nin = S.nman;
    const uint8_t *__restrict__ Min = S.mask;
    float *__restrict__ Hout = S.h[1 - buf];
    float *__restrict__ Uout = S.um[1 - buf];
    float *__restrict__ Vout = S.vn[1 - buf];

    float a_rain = 0.f, a_src = 0.f, a_ev = 0.f, a_out = 0.f, a_clamp = 0.f, cm = 0.f;
    bool bad = false;

    const int unit = blockIdx.x * NWARP + wid;
    if (unit < SH.units) {
        const int ct = unit % SH.tiles_w, rs = unit / SH.tiles_w;
        const int gj0 = ct * kStreamOut - kStreamHL;
        const int gj = gj0 + lane;
        const int R0 = rs * SH.strip_h;
        const int R1 = min(R0 + SH.strip_h, rows);
        const bool out_col = lane >= kStreamHL && lane < kStreamHL + kStreamOut && gj < cols;
        const bool col_cell = (unsigned)gj < (unsigned)cols;
        const bool col_vn = (unsigned)gj <= (unsigned)cols;

        // point sources inside this warp's window, in list order (the later
        // one wins on a shared cell, as the reference's assignment, cu:545)
        int nsrc = 0;
        if (G.n_src > 0) {
            const double area = G.dx * G.dy;
            for (int base = 0; base < G.n_src; base += 32) {
                const int s = base + lane;
                bool in = false;
                int sr = 0, sc = 0;
                if (s < G.n_src) {
                    const int cell = F.src_cell[s];
                    sr = cell / cols;
                    sc = cell - sr * cols;
                    in = sr >= R0 - 4 && sr < R1 + 3 && sc >= gj0 && sc < gj0 + 32;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, in);
                if (in) {
                    const int off = nsrc + __popc(bal & ((1u << lane) - 1u));
                    if (off < kStreamMaxSrc) {
                        s_sr[wid][off] = sr;
                        s_sc[wid][off] = sc;
                        s_q0[wid][off] = (float)source_rate(F, G.n_src, s, ci.plan.t0, area);
                        s_q1[wid][off] = (float)source_rate(F, G.n_src, s, ci.plan.t1, area);
                    } else {
                        atomicOr(&clk[slot_out].status, (unsigned)ST_TOO_MANY_LOCAL_SOURCES);
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
                if (s_sr[wid][e] == row && s_sc[wid][e] == gj) q = second ? s_q1[wid][e] : s_q0[wid][e];
            return q;
        };
        auto storm_rate = [&](int row, bool on, float sx, float sy) -> float {
            if (!on) return 0.f;
            const float x = ((float)gj + 0.5f) * dx - sx;
            const float y = ((float)row + 0.5f) * dy - sy;
            return GS.storm_amp * __expf(-(x * x + y * y) / GS.storm_2s2);
        };

        // row loads (zero outside the domain: inactive, walls)
        float p_h, p_z, p_n, p_um, p_vn;
        unsigned p_m;
        auto load_row = [&](int r) {
            const bool rc = (unsigned)r < (unsigned)rows;
            const size_t gp = (size_t)r * pitch + gj;
            const bool cell = rc && col_cell;
            p_h = cell ? Hin[gp] : 0.f;
            p_z = cell ? Zin[gp] : 0.f;
            p_n = (cell && raster) ? Nin[gp] : manning;
            p_m = cell ? (unsigned)Min[gp] : 0u;
            p_um = ((unsigned)r <= (unsigned)rows && col_cell) ? Uin[gp] : 0.f;
            p_vn = (rc && col_vn) ? Vin[gp] : 0.f;
        };

        // register rings: suffix = rows back from the row being read (r)
        float h1 = 0.f, h2 = 0.f, h3 = 0.f, hL1 = 0.f;
        float z1 = 0.f, z2 = 0.f, zL1 = 0.f;
        float n1 = manning, n2 = manning, nL1 = manning;
        float um1 = 0.f, um2 = 0.f, vn1 = 0.f, vn2 = 0.f;
        float uu_1 = 0.f, uu_2 = 0.f, uuL_1 = 0.f;
        float vv_1 = 0.f, vv_2 = 0.f, vvR_2 = 0.f;
        float rum_2 = 0.f, rum_3 = 0.f, rvn_2 = 0.f, rvn_3 = 0.f;
        float hs_3 = 0.f, hs_4 = 0.f, hw_4 = 0.f;
        unsigned mb = 0u, mLb = 0u;  // bit k: active mask of row r-k (own / west column)

        const int r_first = R0 - 4, r_last = R1 + 3;
        load_row(r_first);
#pragma unroll UNROLL
        for (int r = r_first; r < r_last; r++) {
            const float h0 = p_h, z0 = p_z, n0 = p_n, um0 = p_um, vn0 = p_vn;
            mb = (mb << 1) | p_m;
            const unsigned mL0 = __shfl_up_sync(0xffffffffu, p_m, 1);
            mLb = (mLb << 1) | mL0;
            if (r + 1 < r_last) load_row(r + 1);  // prefetch

            const float hL0 = shup(h0), zL0 = shup(z0);
            const float nL0 = raster ? shup(n0) : manning;
            // ---- row r: face velocities (cu:363-453) ----
            const float hnf = (gj == cols) ? hL0 : ((gj == 0) ? h0 : 0.50f * (h0 + hL0));
            const float vv_0 = (hnf >= ge_th) ? vn0 / hnf : 0.0f;
            const float hmf = (r == rows) ? h1 : ((r == 0) ? h0 : 0.50f * (h0 + h1));
            const float uu_0 = (hmf >= ge_th) ? um0 / hmf : 0.0f;
            const float uuL_0 = shup(uu_0);
            const float vvR_1 = shdn(vv_1);

            // ---- row r-1: new face discharges (cu:98-354) ----
            const int i = r - 1;
            const float umE = shdn(um1), umW = shup(um1);
            const float vnE = shdn(vn1), vnW = shup(vn1);
            const float vvW = shup(vv_1);
            float rum_1 = 0.f;
            if (col_cell) {
                if (i > 0 && i < rows) {
                    const float ha = h2, hb = h1, za = z2, zb = z1;
                    if (((mb >> 2) & (mb >> 1) & 1u) && ((ha >= gt_th) || (hb >= gt_th))) {
                        if (!dry_bed<float>(T, g, ha, za, hb, zb, rum_1)) {
                            const float hm = 0.50f * (hb + ha);
                            const float u13 = g * hm * dt2dx * (hb + zb - ha - za);  // cu:166
                            const float u11uur = 0.50f * (uu_0 + uu_1);
                            const float u11uul = 0.50f * (uu_1 + uu_2);
                            const float u11 = dt2dx * (upwind<float>(u11uur, um0, um1) - upwind_r<float>(u11uul, um2, um1));
                            float u12 = 0.f;  // zero on column 0 (cu:178-180)
                            if (gj != 0) {
                                const float u12vvu = 0.50f * (vvR_1 + vvR_2);
                                const float u12vvd = 0.50f * (vv_1 + vv_2);
                                u12 = dt2dy * (upwind<float>(u12vvu, umE, um1) - upwind_r<float>(u12vvd, umW, um1));
                            }
                            const float rn = 0.5f * (n1 + n2);
                            float ram = 0.f;
                            if ((hm >= gt_th) && rn != 0.f) {  // cu:194-199
                                const float vva = 0.250f * (vv_1 + vvR_1 + vv_2 + vvR_2);
                                ram = g * rn * rn * sqrtf(uu_1 * uu_1 + vva * vva) / RT<float>::pow_(hm);
                            }
                            rum_1 = ((1.00f - dt2 * ram * 0.50f) * um1 + (-u11 - u12 - u13)) /
                                    (1.00f + dt2 * ram * 0.50f);  // cu:203
                        }
                    }
                } else if (i == rows && G.south_open) {  // free outfall (extension)
                    if (((mb >> 2) & 1u) && h2 >= gt_th) rum_1 = 0.5440f * h2 * sqrtf(g * h2);
                }
            }
            float rvn_1 = 0.f;
            if ((unsigned)i < (unsigned)rows && gj > 0 && gj < cols) {
                const float ha = hL1, hb = h1, za = zL1, zb = z1;
                if (((mLb >> 1) & (mb >> 1) & 1u) && ((ha >= gt_th) || (hb >= gt_th))) {
                    if (!dry_bed<float>(T, g, ha, za, hb, zb, rvn_1)) {
                        const float hn = 0.50f * (hb + ha);
                        const float v13 = g * hn * dt2dy * (hb + zb - ha - za);  // cu:283
                        float v11 = 0.f;                                         // zero on row 0 (cu:289-291)
                        if (i != 0) {
                            const float v11uur = 0.50f * (uu_0 + uuL_0);
                            const float v11uul = 0.50f * (uu_1 + uuL_1);
                            v11 = dt2dx * (upwind<float>(v11uur, vn0, vn1) - upwind_r<float>(v11uul, vn2, vn1));
                        }
                        const float v12vvu = 0.50f * (vvR_1 + vv_1);
                        const float v12vvd = 0.50f * (vv_1 + vvW);
                        const float v12 = dt2dy * (upwind<float>(v12vvu, vnE, vn1) - upwind_r<float>(v12vvd, vnW, vn1));
                        const float rn = 0.5f * (n1 + nL1);
                        float ram = 0.f;
                        if ((hn >= gt_th) && rn != 0.f) {  // cu:311-316
                            const float uua = 0.250f * (uu_1 + uu_0 + uuL_1 + uuL_0);
                            ram = g * rn * rn * sqrtf(uua * uua + vv_1 * vv_1) / RT<float>::pow_(hn);
                        }
                        rvn_1 = ((1.00f - dt2 * ram * 0.50f) * vn1 + (-v11 - v12 - v13)) /
                                (1.00f + dt2 * ram * 0.50f);  // cu:320
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
                const float evapo = hi ? LS.ev0 : 0.f;
                const float ql = nsrc ? source_at(r - 2, false) : 0.f;
                const float rr = storm ? storm_rate(r - 2, on0, LS.sx0, LS.sy0) : LS.rr0;
                hs_2 = fmaxf(ho - dt2 * ((rum_1 - rum_2) * rdx + (rvnE_2 - rvn_2) * rdy - ql - rr * pct + evapo), 0.f);
            }

            // ---- row r-3: dry-cell fix (cu:695-725) and final depth ----
            const float hsW_3 = shup(hs_3);
            const bool m3 = (mb >> 3) & 1u, m4 = (mb >> 4) & 1u, m2 = (mb >> 2) & 1u, mL3 = (mLb >> 3) & 1u;
            float un = rum_3;  // x-face north of the row-(r-3) cell
            if ((un > 0.f && m4 && !(hs_4 >= ge_th)) || (un < 0.f && m3 && !(hs_3 >= ge_th))) un = 0.f;
            float us = rum_2;  // x-face south of it
            if ((us > 0.f && m3 && !(hs_3 >= ge_th)) || (us < 0.f && m2 && !(hs_2 >= ge_th))) us = 0.f;
            float vw = rvn_3;  // y-face west of it
            if ((vw > 0.f && mL3 && !(hsW_3 >= ge_th)) || (vw < 0.f && m3 && !(hs_3 >= ge_th))) vw = 0.f;
            const float ve = shdn(vw);
            const int f = r - 3;
            float hw_3 = 0.f, hraw = 0.f, rr1 = 0.f, pct1 = 0.f, ev1 = 0.f, ql1 = 0.f;
            if (m3) {
                const float ho = h3;
                const bool hi = ho >= gt_ev;
                pct1 = hi ? pct_hi : pct_lo;
                ev1 = hi ? LS.ev1 : 0.f;
                ql1 = nsrc ? source_at(f, true) : 0.f;
                rr1 = storm ? storm_rate(f, on1, LS.sx1, LS.sy1) : LS.rr1;
                hraw = ho - dt2 * ((us - un) * rdx + (ve - vw) * rdy - ql1 - rr1 * pct1 + ev1);
                hw_3 = fmaxf(hraw, 0.f);
            }
            const float hwW = shup(hw_3);
            if (out_col && f >= R0 && f < R1) {
                const size_t gp = (size_t)f * pitch + gj;
                Hout[gp] = hw_3;
                Uout[gp] = un;
                Vout[gp] = vw;
                if (f == rows - 1) {
                    Uout[gp + pitch] = us;
                    a_out += us;
                }
                if (m3) {
                    a_rain += rr1 * pct1;
                    a_src += ql1;
                    a_ev += ev1;
                    if (hraw < 0.f) a_clamp -= hraw;
                    // CFL bound of the new state on the owned faces (extension)
                    if (f > 0 && m4) {
                        const float hm = 0.50f * (hw_3 + hw_4);
                        if (hm >= ge_th) cm = fmaxf(cm, fabsf(un / hm) + sqrtf(g * hm));
                    }
                    if (f == rows - 1 && G.south_open && hw_3 >= ge_th)
                        cm = fmaxf(cm, fabsf(us / hw_3) + sqrtf(g * hw_3));
                    if (gj > 0 && mL3) {
                        const float hn = 0.50f * (hw_3 + hwW);
                        if (hn >= ge_th) cm = fmaxf(cm, fabsf(vw / hn) + sqrtf(g * hn));
                    }
                }
                if (!isfinite(hw_3) || !isfinite(un) || !isfinite(vw)) bad = true;
            }

            // ---- advance the rings ----
            h3 = h2; h2 = h1; h1 = h0; hL1 = hL0;
            z2 = z1; z1 = z0; zL1 = zL0;
            n2 = n1; n1 = n0; nL1 = nL0;
            um2 = um1; um1 = um0; vn2 = vn1; vn1 = vn0;
            uu_2 = uu_1; uu_1 = uu_0; uuL_1 = uuL_0;
            vv_2 = vv_1; vv_1 = vv_0; vvR_2 = vvR_1;
            rum_3 = rum_2; rum_2 = rum_1; rvn_3 = rvn_2; rvn_2 = rvn_1;
            hs_4 = hs_3; hs_3 = hs_2;
            hw_4 = hw_3;
        }
    }

    // ---- warp, then CTA reductions; one thread accumulates and finishes ----
    float vals[B_N + 1] = {a_rain, a_src, a_ev, a_out, a_clamp, cm};
#pragma unroll
    for (int q = 0; q < B_N; q++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) vals[q] += __shfl_xor_sync(0xffffffffu, vals[q], o);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vals[B_N] = fmaxf(vals[B_N], __shfl_xor_sync(0xffffffffu, vals[B_N], o));
    const bool wbad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q <= B_N; q++) s_red[wid][q] = vals[q];
        s_bad[wid] = wbad;
    }
    __syncthreads();
    if (tid != 0) return;
    double acc[B_N] = {0, 0, 0, 0, 0};
    float cmb = 0.f;
    bool anybad = false;
    for (int w = 0; w < NWARP; w++) {
        for (int q = 0; q < B_N; q++) acc[q] += (double)s_red[w][q];
        cmb = fmaxf(cmb, s_red[w][B_N]);
        anybad |= s_bad[w] != 0;
    }
    const double area = G.dx * G.dy, scale = ci.plan.d.dt2 * area;
    double v[B_N];
    v[B_RAIN] = acc[B_RAIN] * scale;
    v[B_SRC] = acc[B_SRC] * scale;
    v[B_EV] = acc[B_EV] * scale;
    v[B_OUT] = acc[B_OUT] * ci.plan.d.dt2 * G.dy;
    v[B_CLAMP] = acc[B_CLAMP] * area;
    accumulate_slot(clk[slot_out], blockIdx.x % kBuckets, v, (double)cmb, anybad);
    finish_cta(ci, clk[slot_out], clk[slot_nx], ci.plan, *ctl, G, F);
}

}  // namespace sw2d
