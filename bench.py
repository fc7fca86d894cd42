"""Benchmark of the SW2D time-stepping core on GB300.

Workload (the synthetic-catchment configuration): a 2048 x 2048 grid, dx = 5 m,
DEM = tilted plane (slope 0.01 toward the south edge) + seeded 6-octave fractal
noise (amplitude 2 m, persistence 0.5) + a 3-cell carved channel, Manning n
from 4 land-use classes by seeded Voronoi patches, uniform rain 50 mm/h for
t < 3600 s, open south edge, CFL 0.5.  The state is spun up (untimed) to
t = 1800 s, mid-storm, when every active cell is wet.

One bench step = one replay of the CUDA graph of 48 solver iterations (each
iteration advances every cell by one time step Dt = 2 dt).  Metric:
cell-updates/s = active cells x iterations / time.  The L2 cache (129 MB) is
flushed between bench steps by writing a 256 MB buffer on the solver's stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU oracle (the serial C restatement of the
reference update, OpenMP over rows, FP64) on the host cores, on a bounded
sample of the same workload.  Under torchrun every rank runs an independent
replica on its own GPU (the scenarios share nothing), rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sw2d-gpu_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CHUNK = 48               # solver iterations per bench step (one graph replay)
SIZE = 2048
DX = 5.0
SEED = 20240
RAIN_MM_H = 50.0
RAIN_HOURS = 1.0
SPINUP_T = 1800.0
DT_MAX = 1.0             # largest half step [s]
B_ALG_F32 = 32           # algorithmic bytes per cell-update: read h,um,vn,z,n + write h,um,vn (FP32)
B_ALG_F64 = 64
METRIC = "cell-updates/s"
ACC_WINDOW_S = 60.0      # simulated seconds of the FP32-vs-FP64 accuracy leg
LARGE = 8192             # the large-single-domain configuration: 8192^2, dx 2 m, n 0.05, moving storm
LARGE_DX = 2.0
LARGE_SPINUP_T = 1800.0  # the storm centre has crossed most of the diagonal by then
B_ALG_F32_SCALAR_N = 28  # algorithmic bytes per cell-update with a scalar Manning n


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def scenario(seed):
    from sw2d import scenarios as S
    return S.catchment(SIZE, dx=DX, seed=seed)


def make_solver(sw2d, s, precision, device):
    g = sw2d.Solver(rows=SIZE, cols=SIZE, dx=DX, dy=DX, precision=precision, dt_mode=sw2d.DT_CFL, dt=DT_MAX,
                    cfl=0.5, south_open=1, device=device)
    g.set_static(s["z"], s["n"])
    g.set_rain(sw2d.RAIN_STEP, [RAIN_MM_H] * int(RAIN_HOURS), 3600.0)
    return g


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def steps_per_launch(desc):
    """Iterations per kernel launch of a solver, from its sw2d_describe line."""
    for tok in desc.split():
        if tok.startswith("steps_per_launch="):
            return int(tok.split("=")[1])
    return 1


def traffic_per_cell_update():
    """DRAM bytes per cell-update of the FP32 step kernel from the committed
    ncu summary (dram__bytes_read.sum + dram__bytes_write.sum of one launch
    divided by the cells it updates), or None."""
    p = os.path.join(ROOT, "profiles", "step_f32_catchment.dram.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_cell_update:"):
            return float(line.split(":")[1])
    return None


def run_ours(args):
    import numpy as np
    import torch
    import sw2d

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = local
    torch.cuda.set_device(dev)
    sw2d.load()
    from sw2d import autotune, replicas
    s = scenario(replicas.rank_seed(SEED, rank))
    active = int(np.count_nonzero(s["z"] != -9999.0))

    # ---- autotuning (untimed): strip height and kernel build of the
    # single-domain kernel for this size class, build and graph chunk of the
    # batched kernel; the solvers and batches below take the choices.  The
    # cache lives beside the built library, so a fresh build tunes afresh.
    os.environ.setdefault("SW2D_AUTOTUNE_CACHE", os.path.join(ROOT, "sw2d-gpu_gb300", "_build", "autotune.json"))
    t_tune = time.perf_counter()
    tuned = autotune.tune(SIZE, SIZE, device=dev, iters=CHUNK, strips=())
    tuned_b = autotune.tune_batch(device=dev) if (args.batched or args.served) else {}
    tune_s = time.perf_counter() - t_tune
    log(f"[rank {rank}] autotune: strip_h={tuned['strip_h']} variant={tuned['variant']} "
        f"batch={tuned_b.get('variant')}/{tuned_b.get('chunk')}/{tuned_b.get('strip_h')} ({tune_s:.1f}s, "
        f"{len(tuned.get('timings', []))} + {len(tuned_b.get('timings', []))} candidates)")

    g = make_solver(sw2d, s, sw2d.PREC_F32, dev)
    g.set_state(s["h0"])
    t0 = time.time()
    g.advance(10 ** 9, t_end=SPINUP_T)
    log(f"[rank {rank}] spin-up to t={SPINUP_T}s: {g.budget()['steps']} iterations, {time.time() - t0:.1f}s wall")
    spun = g.state()

    stream = torch.cuda.ExternalStream(g.stream())
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{dev}")

    def timed_chunks(solver, k, w, per_chunk=CHUNK, counts=None):
        st = torch.cuda.ExternalStream(solver.stream())
        for _ in range(w):
            solver.advance(per_chunk)
        times = []
        launches0 = solver.launch_count()
        for _ in range(k):
            with torch.cuda.stream(st):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            n = solver.advance(per_chunk)
            e1.record(st)
            e1.synchronize()
            assert n == per_chunk, f"advance stopped after {n} iterations"
            times.append(e0.elapsed_time(e1) / 1e3)
        if counts is not None:
            counts["launches"] = solver.launch_count() - launches0
        return times

    # ---- device-timed FP32 (the product path) -------------------------------
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev)
    sampler.start()
    wall0 = time.perf_counter()
    counts = {}
    times = timed_chunks(g, args.steps, args.warmup, counts=counts)
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    torch.cuda.synchronize()
    launches = counts["launches"]  # the library's kernels issued by the timed advances
    local_s = sum(times)
    cu_all, tot = replicas.job_totals(active * CHUNK * args.steps, local_s, device=f"cuda:{dev}")
    value = cu_all / tot  # units of all ranks / seconds of the slowest rank
    per_launch = local_s / (CHUNK * args.steps)
    peak, peak_kind = peaks()
    achieved = B_ALG_F32 * active / per_launch / 1e9
    tpc = traffic_per_cell_update()
    kernel_desc = g.describe()
    bud = g.budget()
    vol_err = abs(bud["volume"] - (bud["volume0"] + bud["rain_in"] + bud["source_in"] - bud["evap_out"] -
                                   bud["outflow"] + bud["clamp_gain"])) / max(bud["volume"], 1e-30)
    g.close()

    # ---- FP64 plain path on the same spun-up state (secondary) -------------
    g64 = make_solver(sw2d, s, sw2d.PREC_F64, dev)
    g64.set_state(spun["h"], spun["um"], spun["vn"], t0=SPINUP_T)
    t64 = timed_chunks(g64, max(2, args.steps // 40), 1)
    v64 = active * CHUNK * len(t64) / sum(t64)
    g64.close()

    # ---- error of the FP32 path against FP64 on this workload ---------------
    accuracy = fp32_vs_fp64(sw2d, s, spun, dev)

    # ---- end to end through the C ABI with host buffers ----------------------
    # as many advances as timed steps and at least 20, so that the one-time
    # upload is amortised over a run of some length whatever --steps is
    k_e2e = max(20, args.steps)
    h_pinned = torch.from_numpy(s["h0"]).pin_memory()
    z_pinned = torch.from_numpy(s["z"]).pin_memory()
    n_pinned = torch.from_numpy(s["n"]).pin_memory()
    spun_pin = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in spun.items()}
    torch.cuda.synchronize()
    te0 = time.perf_counter()
    ge = sw2d.Solver(rows=SIZE, cols=SIZE, dx=DX, dy=DX, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_CFL, dt=DT_MAX,
                     cfl=0.5, south_open=1, device=dev)
    ge.set_static(z_pinned.numpy(), n_pinned.numpy())
    ge.set_rain(sw2d.RAIN_STEP, [RAIN_MM_H], 3600.0)
    ge.set_state(spun_pin["h"].numpy(), spun_pin["um"].numpy(), spun_pin["vn"].numpy(), t0=SPINUP_T)
    for _ in range(k_e2e):
        ge.advance(CHUNK)
        ge.budget()  # device->host read of the step's result (volume + budgets)
    out_h = ge.depth()
    te = time.perf_counter() - te0
    ge.close()
    del h_pinned
    e2e_value = active * CHUNK * k_e2e / te
    # bytes the library copies (sw2d_api.cu): set_static z, n; set_state h, um, vn and the
    # initial clock slot, then one clock read and one budget read (1024 volume partials);
    # the rain table; per advance one Control down and one clock slot up; per budget the
    # volume partials; the final depth
    clock_b, control_b, partials_b = 1120, 16, 1024 * 8
    h2d = (SIZE * SIZE * 8) * 3 + ((SIZE + 1) * SIZE * 8) * 2 + clock_b + 8 + k_e2e * control_b
    d2h = (clock_b + partials_b) + k_e2e * (clock_b + partials_b) + SIZE * SIZE * 8
    assert np.isfinite(out_h).all()

    # ---- large single domain (extra key) -------------------------------------
    large = run_large(sw2d, dev, args, peak) if args.large else None

    # ---- batched ensemble and served stream (extra keys) --------------------
    batched = run_batched(sw2d, dev, args, rank, ws) if args.batched else None
    served = run_served(sw2d, dev, args) if args.served else None
    served_sweep = None
    if args.serve_sweep:
        served_sweep = []
        for rate in (float(x) for x in args.serve_sweep.split(",")):
            args.serve_rate = rate
            served_sweep.append(run_served(sw2d, dev, args))

    # ---- CPU baseline: the oracle on a bounded sample ------------------------
    cpu = cpu_sample(s, spun, budget_s=args.cpu_seconds) if rank == 0 else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "synthetic catchment 2048x2048, dx 5 m, rain 50 mm/h, open south edge, CFL 0.5, "
                                   "state spun up to t=1800 s; FP32 state, FP64 budgets",
                       "grid": [SIZE, SIZE], "active_cells": active, "iterations_per_step": CHUNK,
                       "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{ws}",
                       "seed": SEED,
                       "autotuned": {"strip_h": tuned["strip_h"], "variant": tuned["variant"], "kernel": kernel_desc,
                                     "batch_variant": tuned_b.get("variant"), "batch_chunk": tuned_b.get("chunk"),
                                     "batch_strip_h": tuned_b.get("strip_h"),
                                     "steps_per_launch": steps_per_launch(kernel_desc), "tuning_s": tune_s,
                                     "candidates": len(tuned.get("timings", [])) + len(tuned_b.get("timings", []))}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": (tpc * active if tpc is not None else None),
                         "bytes_alg_per_cell_update": B_ALG_F32, "kernel": kernel_desc,
                         "launch_s": per_launch},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d / k_e2e,
                    "d2h_bytes_per_step": d2h / k_e2e, "steps": k_e2e},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "wall_s_timed": wall,
            "fp64_plain": {"value": v64, "unit": "cell-updates/s", "speedup_f32_over_f64": value / ws / v64},
            "volume_rel_error": vol_err,
            "accuracy_vs_fp64": accuracy,
            "large_domain": large,
            "batched": batched,
            "served": served,
        }
        if served_sweep is not None:
            line["served_sweep"] = served_sweep
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


_BANK = None


def terrain_bank():
    global _BANK
    if _BANK is None:
        from sw2d import scenarios as S
        _BANK = S.TerrainBank(size=SIZE, dx=DX, seed=SEED + 7)
    return _BANK


def scen_cfg(sw2d, side, precision=None, device=0):
    return sw2d.default_config(rows=side, cols=side, dx=DX, dy=DX,
                               precision=sw2d.PREC_F32 if precision is None else precision,
                               dt_mode=sw2d.DT_CFL, dt=DT_MAX, cfl=0.5, south_open=1, device=device)


def depth_error(a, b, th=1.0e-4):
    """max |dh| [m], its 99.99th percentile and the flooded-area (h > th)
    relative difference of depth rasters a (FP64) and b."""
    d = np.abs(a - b)
    wa, wb = int(np.count_nonzero(a > th)), int(np.count_nonzero(b > th))
    return {"max_abs_dh_m": float(d.max()), "p9999_abs_dh_m": float(np.percentile(d, 99.99)),
            "cells_over_1mm": int(np.count_nonzero(d > 1e-3)), "cells": int(d.size),
            "flooded_area_rel_diff": abs(wa - wb) / max(wa, 1)}


def fp32_vs_fp64(sw2d, s, spun, dev, window=ACC_WINDOW_S):
    """FP32 and FP64 advanced from the same spun-up state to the same
    simulated time (each with its own CFL steps); the depth error of FP32,
    and beside it the FP64 run's own response to the rain rate raised by one
    part in a million (the conditioning of the flow over the window)."""
    out = {}
    for key, prec, scale in (("f64", sw2d.PREC_F64, 1.0), ("f32", sw2d.PREC_F32, 1.0),
                             ("f64_rain_1e-6", sw2d.PREC_F64, 1.0 + 1e-6)):
        g = make_solver(sw2d, s, prec, dev)
        g.set_rain(sw2d.RAIN_STEP, [RAIN_MM_H * scale], RAIN_HOURS * 3600.0)
        g.set_state(spun["h"], spun["um"], spun["vn"], t0=SPINUP_T)
        g.advance(10 ** 9, t_end=SPINUP_T + window)
        out[key] = (g.depth(), g.budget())
        g.close()
    e = depth_error(out["f64"][0], out["f32"][0])
    e.update({"window_s": window, "from_t_s": SPINUP_T, "steps_fp64": int(out["f64"][1]["steps"]),
              "steps_fp32": int(out["f32"][1]["steps"]),
              "fp64_vs_fp64_rain_1e-6": depth_error(out["f64"][0], out["f64_rain_1e-6"][0])})
    return e


def run_batched(sw2d, dev, args, rank=0, ws=1):
    """The batched-ensemble configuration: 256 scenarios, sides uniform over
    {128, 256, 512, 1024}, triangular hyetographs, Manning scaling, horizon =
    rain duration + 1800 s; all advanced together until the last one ends.
    The serial FP64 plain path is measured on whole scenarios of every size
    class (fp64_alone).  Under torchrun each rank advances its contiguous
    share of the ensemble."""
    import torch
    from sw2d import replicas
    from sw2d import scenarios as S
    ens_all = S.ensemble(terrain_bank(), count=args.batch_count, seed=SEED + 11)
    ens = [ens_all[k] for k in replicas.shard(len(ens_all), rank, ws)]
    t0 = time.perf_counter()
    b = sw2d.Batch(device=dev, max_scenarios=len(ens) + 8)  # build, chunk and strip height: the autotuner's
    ids = [b.add(scen_cfg(sw2d, e["side"], device=dev), e["z"], e["h0"], manning=e["n"],
                 rain_kind=sw2d.RAIN_LINEAR, rain=e["rain"], rain_dt=e["rain_dt"], t_end=e["t_end"]) for e in ens]
    t_admit = time.perf_counter() - t0
    st = torch.cuda.ExternalStream(b.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    launches0 = b.launch_count()
    running = len(ids)
    while running:
        running = b.advance(48)
    e1.record(st)
    e1.synchronize()
    gpu_s = e0.elapsed_time(e1) / 1e3
    wall = time.perf_counter() - t0
    status = b.poll()
    cu = sum(e["side"] * e["side"] * status[i]["steps"] for e, i in zip(ens, ids))
    launches = b.launch_count() - launches0
    # The serial baseline, measured: the FP64 plain single-scenario path runs
    # `batch_fp64_per_class` whole scenarios of each size class one after the
    # other, each alone to its own end time (set-up, advance and the depth
    # download timed); each result is also the FP64 reference of the batched
    # FP32 result of the same scenario.  The serial time of the whole ensemble
    # is each class's mean measured time times the class's scenario count.
    by_side = {}
    for k, e in enumerate(ens):
        by_side.setdefault(e["side"], []).append(k)
    # Beside the error of FP32, the conditioning of the scenario where it is
    # largest: the FP64 result's own change when the rain is raised by one
    # part in a million.  Wet/dry thresholds and the dry-bed rules switch
    # discontinuously, so over hours of simulated time the pointwise solution
    # moves by millimetres under perturbations far below FP32 rounding.
    measured, errors = {}, []
    for side in sorted(by_side):
        errs, h64s = [], []
        for k in by_side[side][:args.batch_fp64_per_class]:
            sec, h64, _ = fp64_alone(sw2d, dev, ens[k])
            measured.setdefault(side, []).append(sec)
            errs.append(depth_error(h64, b.field(ids[k], sw2d.FIELD_DEPTH)))
            h64s.append(h64)
        w = max(range(len(errs)), key=lambda n: errs[n]["max_abs_dh_m"])
        k = by_side[side][w]
        sens = depth_error(h64s[w], fp64_alone(sw2d, dev, ens[k], rain_scale=1.0 + 1e-6)[1])
        errors.append({"side": side, "scenarios": len(errs),
                       "max_abs_dh_m": max(x["max_abs_dh_m"] for x in errs),
                       "p9999_abs_dh_m": max(x["p9999_abs_dh_m"] for x in errs),
                       "cells_over_1mm": sum(x["cells_over_1mm"] for x in errs),
                       "flooded_area_rel_diff": max(x["flooded_area_rel_diff"] for x in errs),
                       "worst_scenario": {"index": k, "fp32_vs_fp64": errs[w], "fp64_vs_fp64_rain_1e-6": sens}})
    b.close()
    serial64_meas = sum(statistics.mean(measured[side]) * len(by_side[side]) for side in by_side)
    # the earlier estimate beside it: the FP64 rate on a 5 mm film per size
    # class times the ensemble's own FP32 iteration counts
    rate64 = {}
    for side in sorted(by_side):
        e = ens[by_side[side][0]]
        g = sw2d.Solver(scen_cfg(sw2d, side, precision=sw2d.PREC_F64, device=dev))
        g.set_static(e["z"], e["n"])
        g.set_state(np.full((side, side), 0.005))
        g.set_rain(sw2d.RAIN_LINEAR, e["rain"], e["rain_dt"])
        g.advance(6)
        g.synchronize()
        tt = time.perf_counter()
        n = g.advance(max(6, int(2e8 / (side * side))))
        g.synchronize()
        rate64[side] = side * side * n / (time.perf_counter() - tt)
        g.close()
    serial64_s = sum(e["side"] * e["side"] * status[i]["steps"] / rate64[e["side"]] for e, i in zip(ens, ids))
    dev_name = f"cuda:{dev}"
    cu_all, gpu_s_all = replicas.job_totals(cu, gpu_s, device=dev_name)
    n_all, wall_all = replicas.job_totals(len(ens), wall, device=dev_name)
    serial_all, _ = replicas.job_totals(serial64_s, 0.0, device=dev_name)
    serial_meas_all, _ = replicas.job_totals(serial64_meas, 0.0, device=dev_name)
    return {"scenarios": int(n_all), "cells": int(sum(e["side"] ** 2 for e in ens_all)), "cell_updates": int(cu_all),
            "gpu_s": gpu_s_all, "wall_s_incl_admission": wall_all, "admission_s": t_admit, "launches": int(launches),
            "cell_updates_per_s": cu_all / gpu_s_all, "scenarios_per_hour": n_all / wall_all * 3600.0,
            "serial_fp64_s": serial_meas_all,
            "serial_fp64_measured": {str(k): {"scenarios": len(v), "seconds": v,
                                              "of_class": len(by_side[k])} for k, v in measured.items()},
            "serial_fp64_how": (f"{args.batch_fp64_per_class} whole scenarios per size class run alone through the "
                                "FP64 plain path to their own end times; class mean x class count"),
            "scenario_throughput_vs_serial_fp64": serial_meas_all / wall_all,
            "serial_fp64_plain_s_est": serial_all, "fp64_plain_rate_by_side": {str(k): v for k, v in rate64.items()},
            "horizon": "rain duration + 1800 s", "ranks": ws, "accuracy_vs_fp64": errors}


def run_large(sw2d, dev, args, peak):
    """The large-single-domain configuration: 8192 x 8192 cells of 2 m, the
    catchment DEM with uniform n = 0.05, a Gaussian storm cell (80 mm/h,
    sigma 2 km) moving at 10 m/s from the north-west corner along the
    diagonal, open south edge, CFL 0.5.  Spun up in FP32 to t = 1800 s, then
    `large_steps` windows of 48 iterations timed with CUDA events on the
    solver's stream, L2 flushed between windows; the FP64 path then runs the
    same simulated interval from the same state for the error of the FP32
    result."""
    import torch
    from sw2d import large_domain as LD
    from sw2d import scenarios as S
    t0 = time.perf_counter()
    s = S.catchment(LARGE, dx=LARGE_DX, seed=3, manning=0.05)
    st = LD.storm_params(LARGE, LARGE_DX)

    def solver(prec):
        g = sw2d.Solver(rows=LARGE, cols=LARGE, dx=LARGE_DX, dy=LARGE_DX, precision=prec, dt_mode=sw2d.DT_CFL,
                        dt=DT_MAX, cfl=0.5, south_open=1, manning=0.05, device=dev)
        g.set_static(s["z"])
        g.set_storm(st["peak"], st["x0"], st["y0"], st["vx"], st["vy"], st["sigma"])
        return g

    g = solver(sw2d.PREC_F32)
    g.set_state(s["h0"])
    g.advance(10 ** 9, t_end=LARGE_SPINUP_T)
    t_start = g.budget()["t"]
    strm = torch.cuda.ExternalStream(g.stream())
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{dev}")
    g.advance(CHUNK)  # warm-up window (graph instantiation)
    g.synchronize()
    t_from = g.budget()["t"]
    from_state = g.state()
    times = []
    for _ in range(args.large_steps):
        with torch.cuda.stream(strm):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(strm)
        n = g.advance(CHUNK)
        e1.record(strm)
        e1.synchronize()
        assert n == CHUNK
        times.append(e0.elapsed_time(e1) / 1e3)
    bud = g.budget()
    h32 = g.depth()
    t_end = bud["t"]
    kernel = g.describe()
    g.close()
    del flush
    vol_err = abs(bud["volume"] - (bud["volume0"] + bud["rain_in"] + bud["source_in"] - bud["evap_out"] -
                                   bud["outflow"] + bud["clamp_gain"])) / max(bud["volume"], 1e-30)
    g64 = solver(sw2d.PREC_F64)
    g64.set_state(from_state["h"], from_state["um"], from_state["vn"], t0=t_from)
    n64 = g64.advance(10 ** 9, t_end=t_end)
    h64 = g64.depth()
    g64.close()
    cells = LARGE * LARGE
    per_launch = sum(times) / (CHUNK * len(times))
    rate = cells / per_launch
    err = depth_error(h64, h32)
    err.update({"from_t_s": t_from, "to_t_s": t_end, "iterations_fp32": CHUNK * len(times),
                "iterations_fp64": int(n64)})
    return {"grid": [LARGE, LARGE], "dx": LARGE_DX, "cell_updates_per_s": rate, "launch_s": per_launch,
            "windows": len(times), "iterations_per_window": CHUNK, "spinup_to_t_s": t_start,
            "l2": "flushed between windows (256 MB write)", "kernel": kernel,
            "roofline": {"bound": "hbm", "bytes_alg_per_cell_update": B_ALG_F32_SCALAR_N,
                         "achieved": B_ALG_F32_SCALAR_N * rate / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": B_ALG_F32_SCALAR_N * rate / 1e9 / peak},
            "volume_rel_error": vol_err, "wet_fraction": float(np.mean(h32 > 1.0e-4)),
            "accuracy_vs_fp64": err, "wall_s": time.perf_counter() - t0}


def fp64_alone(sw2d, dev, e, rain_scale=1.0):
    """One scenario through the FP64 plain single-scenario path, alone, to its
    end time: (seconds for set-up, run and depth download, depth, steps)."""
    import torch
    torch.cuda.synchronize()
    tt = time.perf_counter()
    g = sw2d.Solver(scen_cfg(sw2d, e["side"], precision=sw2d.PREC_F64, device=dev))
    g.set_static(e["z"], e["n"])
    g.set_state(e["h0"])
    g.set_rain(sw2d.RAIN_LINEAR, np.asarray(e["rain"]) * rain_scale, e["rain_dt"])
    g.advance(10 ** 9, t_end=e["t_end"])
    h = g.depth()
    steps = g.budget()["steps"]
    sec = time.perf_counter() - tt
    g.close()
    return sec, h, steps


def run_served(sw2d, dev, args):
    """The served-stream configuration at one arrival rate: log-uniform
    sides 64-2048 (multiples of 32), horizons U[600, 7200] s, Poisson
    arrivals; continuous batching with admission by device footprint."""
    from sw2d import scenarios as S
    from sw2d import serve
    specs = S.request_stream(terrain_bank(), rate=args.serve_rate, count=args.serve_count, seed=SEED + 13)
    reqs = [serve.Request(rid=k, arrival=sp["arrival"], cfg=scen_cfg(sw2d, sp["side"], device=dev), z=sp["z"],
                          depth=sp["h0"], manning=sp["n"], rain_kind=sw2d.RAIN_LINEAR, rain=sp["rain"],
                          rain_dt=sp["rain_dt"], t_end=sp["t_end"]) for k, sp in enumerate(specs)]
    budget = int(args.serve_gb * 2 ** 30)
    # a sample of requests, spread over the sides up to 1024, whose served
    # depth is kept for the comparison with the FP64 plain path
    order = sorted((sp["side"], k) for k, sp in enumerate(specs) if sp["side"] <= 1024)
    m = min(args.serve_fp64_sample, len(order))
    sample = {order[int(round(i * (len(order) - 1) / max(m - 1, 1)))][1] for i in range(m)}
    from sw2d import autotune
    bc = autotune.apply_batch(sw2d.batch_config(device=dev))  # the batch build and graph chunk
    tick = bc.chunk  # a tick is one graph replay
    # the library's own serving loop (sw2d_server_*): admission by device
    # footprint and free slots, one tick per step, retirement with the
    # results copied to the host; Python submits each request at its arrival
    srv = serve.NativeServer(lambda: sw2d.ServerHandle(device=dev, max_scenarios=len(reqs) + 8, max_bytes=budget,
                                                       chunk=bc.chunk, variant=bc.variant, launches_per_step=tick,
                                                       keep_depth=1),
                             keep_results=lambda r: r.rid in sample)
    st = srv.run(reqs, timeout=600.0)
    srv.close()
    st.update({"rate_per_s": args.serve_rate, "memory_budget_gb": args.serve_gb, "launches_per_tick": tick,
               "loop": "sw2d_server_* (library)"})
    # the plain sequential FP64 path on the same request set: the sampled
    # requests run alone in FP64 (measured: their time and their error); every
    # other request's FP64 time is its served cell-updates at the FP64 rate
    # measured on the sampled request nearest in side; then a one-at-a-time
    # queue in arrival order gives the sequential path's time to result
    served = {r.rid: r for r in srv.done if r.result and "steps" in r.result}
    meas, errs = [], []
    for k in sorted(sample):
        if k not in served:
            continue
        sec, h64, steps = fp64_alone(sw2d, dev, specs[k])
        side = specs[k]["side"]
        meas.append({"side": side, "seconds": sec, "rate": side * side * steps / sec})
        e = depth_error(h64, served[k].result["depth"])
        e["side"] = side
        errs.append(e)
    if meas:
        def fp64_seconds(r):
            side = int(r.cfg.rows)
            near = min(meas, key=lambda x: abs(np.log(x["side"] / side)))
            return side * side * r.result["steps"] / near["rate"]
        t_free, ttr = 0.0, []
        for r in sorted(served.values(), key=lambda r: r.arrival):
            t_free = max(t_free, r.arrival) + fp64_seconds(r)
            ttr.append(t_free - r.arrival)
        seq_s = sum(fp64_seconds(r) for r in served.values())
        span = max(t_free, st["span_s"])
        st["sequential_fp64"] = {
            "how": (f"{len(meas)} requests (sides {min(x['side'] for x in meas)}-{max(x['side'] for x in meas)}) "
                    "run alone through the FP64 plain path, measured; the others at the FP64 rate of the measured "
                    "request nearest in side; a one-at-a-time queue in arrival order"),
            "measured": meas, "busy_s": seq_s, "p50_s": float(np.percentile(ttr, 50)),
            "p99_s": float(np.percentile(ttr, 99)), "scenarios_per_hour": len(served) / span * 3600.0,
            "served_speedup_scenarios_per_hour": st["scenarios_per_hour"] / (len(served) / span * 3600.0)}
        st["accuracy_vs_fp64"] = {"sample": errs, "max_abs_dh_m": max(e["max_abs_dh_m"] for e in errs),
                                  "max_flooded_area_rel_diff": max(e["flooded_area_rel_diff"] for e in errs)}
    return st


def cpu_sample(s, spun, budget_s=12.0):
    """The CPU oracle on the same workload: the spun-up 2048x2048 state,
    iterated for about `budget_s` seconds with all host threads."""
    import oracle as O
    o = O.Oracle(SIZE, SIZE, DX, DX, s["z"], n=s["n"], dt_mode=1, dt=DT_MAX, cfl=0.5, south_open=1)
    o.set_state(spun["h"], spun["um"], spun["vn"], t=SPINUP_T)
    o.set_forcing(O.OracleForcing(rain_kind=O.RAIN_STEP, rain=[RAIN_MM_H], rain_dt=3600.0))
    active = int((s["z"] != -9999.0).sum())
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        n += o.advance(1)
    el = time.perf_counter() - t0
    return {"value": active * n / el, "unit": "cell-updates/s", "cores": O.max_threads(), "kind": "port",
            "sample": f"{n} iterations of the spun-up 2048x2048 catchment, FP64, {el:.1f} s"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle as O
    O.build()
    s = scenario(SEED)
    o = O.Oracle(SIZE, SIZE, DX, DX, s["z"], n=s["n"], dt_mode=1, dt=DT_MAX, cfl=0.5, south_open=1)
    o.set_forcing(O.OracleForcing(rain_kind=O.RAIN_STEP, rain=[RAIN_MM_H], rain_dt=3600.0))
    # the spin-up is not part of the reference arm's timing: start from a
    # uniform 5 mm film, mid-storm, so that every cell does the full update
    import numpy as np
    o.set_state(np.where(s["z"] != -9999.0, 0.005, 0.0), t=SPINUP_T)
    active = int((s["z"] != -9999.0).sum())
    per_step = 2  # iterations of the full grid per reference bench step (bounded sample)
    for _ in range(args.warmup):
        o.advance(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.advance(per_step)
    el = time.perf_counter() - t0
    value = active * per_step * args.steps / el
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": "synthetic catchment 2048x2048 (the same grid), FP64 reference scheme on host cores",
                   "grid": [SIZE, SIZE], "active_cells": active, "iterations_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": O.max_threads(), "kind": "port",
                         "sample": f"{per_step} iterations of the 2048x2048 catchment per step"},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--batched", type=int, default=1, help="run the batched-ensemble leg")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--large", type=int, default=1, help="run the large-single-domain leg (8192^2, moving storm)")
    ap.add_argument("--large-steps", type=int, default=3, help="timed 48-iteration windows of the large leg")
    ap.add_argument("--served", type=int, default=1, help="run the served-stream leg")
    ap.add_argument("--serve-rate", type=float, default=10.0)
    ap.add_argument("--serve-count", type=int, default=100)
    ap.add_argument("--serve-gb", type=float, default=40.0)
    ap.add_argument("--serve-sweep", default="", help="comma-separated arrival rates, e.g. 2,5,10,20,50")
    ap.add_argument("--batch-fp64-per-class", type=int, default=4,
                    help="whole scenarios per size class run through the FP64 plain path (serial baseline, accuracy)")
    ap.add_argument("--serve-fp64-sample", type=int, default=6,
                    help="served requests rerun alone through the FP64 plain path (sequential baseline, accuracy)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
