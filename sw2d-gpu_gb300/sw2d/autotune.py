"""Autotuner for the FP32 kernels: tile shape, kernel build, iterations per
launch, launches per sync.

For a grid-size class it times every candidate (strip height, kernel build)
of the single-scenario streaming kernel on a wet synthetic catchment of that
size and keeps the fastest; under the reference's fixed time step it also
times the iterations per launch (tune_fixed: one launch per iteration
against 24, 48 and 96 iterations per cooperative launch); for batches it
times the builds of the batched kernel with the CUDA-graph chunk
(iterations replayed between host synchronisations) on a small ensemble.
Results are cached in a JSON file keyed by GPU name and size class
(SW2D_AUTOTUNE_CACHE names the file), so a tuning run is paid once per
machine.  Solver(**kw) and Batch(**kw) take the cached choice when the
caller leaves the decomposition to the library (SW2D_AUTOTUNE=0 turns that
off).

    from sw2d import autotune
    best = autotune.tune(2048, 2048)          # {"strip_h": 52, "variant": 0, ...}
    autotune.tune_fixed(1024, 1024)           # {"strip_h": 0, "variant": 0, "steps_per_launch": 48, ...}
    cfg = autotune.apply(cfg)                 # fills strip_h/variant (and steps_per_launch) from the cache
    autotune.tune_batch()                     # {"variant": 0, "chunk": 24, ...}
"""
from __future__ import annotations

import json
import os
import time
from typing import Callable, Optional

import numpy as np

STRIPS = (16, 24, 32, 48, 64, 96, 128)
VARIANTS = (0, 1, 2, 3, 4, 5)
CHUNKS = (12, 24, 48, 96)
OUT_COLS = 27            # output columns of one streaming warp
RESIDENT_WARPS_PER_SM = (16, 20, 24)  # resident warps per SM of the kernel builds


# Variant ids index the kernel builds of the library; a cache written for
# another table of builds is not reused.
TABLE_VERSION = "stream-v5"


def wave_strips(rows: int, cols: int, sms: int = 152, waves=(1, 2, 3, 4), warps_per_sm=RESIDENT_WARPS_PER_SM):
    """Strip heights that cut every column tile into as many strips as fill
    the resident warps of the GPU in `w` whole waves, for each w and each
    resident-warp count of the kernel builds."""
    tiles_w = -(-cols // OUT_COLS)
    return sorted({max(16, -(-rows // max(1, (w * sms * per) // tiles_w))) for w in waves for per in warps_per_sm})


BATCH_VARIANTS = (0, 1, 2)
# rows per warp for every scenario of a batch (0: by scenario size, 16/32/64
# rows); taller strips repeat fewer warm-up rows, which pays on a large
# ensemble (measured on GB300, 64 scenarios of 128-1024 cells a side: 4.85e10
# cell-updates/s by size, 4.98e10 with 64 rows, 5.02e10 with 96)
BATCH_STRIPS = (0, 64, 96)
BATCH_CLASS = "batch"
STEPS_PER_LAUNCH = (1, 24, 48, 96)  # fixed time step: iterations per launch tried by tune_fixed
FIXED_VARIANTS = (0, 2)


def fixed_class(rows: int, cols: int) -> str:
    """Cache key of the fixed-time-step choices of a size class."""
    return "fixed|" + size_class(rows, cols)


def default_cache_path() -> str:
    if os.environ.get("SW2D_AUTOTUNE_CACHE"):
        return os.environ["SW2D_AUTOTUNE_CACHE"]
    base = os.environ.get("XDG_CACHE_HOME", os.path.join(os.path.expanduser("~"), ".cache"))
    return os.path.join(base, "sw2d", "autotune.json")


def enabled() -> bool:
    return os.environ.get("SW2D_AUTOTUNE", "1") != "0"


def size_class(rows: int, cols: int) -> str:
    """Grids within a factor sqrt(2) in cell count share a class."""
    return f"c{int(round(2 * np.log2(max(rows * cols, 1))))}"


class Cache:
    def __init__(self, path: Optional[str] = None):
        self.path = path or default_cache_path()
        self.data = {}
        if os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    self.data = json.load(f)
            except (OSError, ValueError):
                self.data = {}

    def get(self, gpu: str, cls: str):
        return self.data.get(gpu, {}).get(cls)

    def put(self, gpu: str, cls: str, entry: dict):
        self.data.setdefault(gpu, {})[cls] = entry
        os.makedirs(os.path.dirname(self.path) or ".", exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def gpu_name(device: int = 0) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:
        return "unknown-gpu"


def _sm_count(device: int = 0) -> int:
    try:
        import torch
        return torch.cuda.get_device_properties(device).multi_processor_count
    except Exception:
        return 152


def search(candidates, timer: Callable[[dict], float]):
    """Times every candidate (seconds per iteration, lower is better) and
    returns (best candidate, table of timings)."""
    table = []
    for c in candidates:
        try:
            t = float(timer(c))
        except Exception as e:  # a candidate that cannot run is skipped
            table.append({**c, "error": str(e)})
            continue
        table.append({**c, "s_per_iter": t})
    ok = [r for r in table if "s_per_iter" in r]
    if not ok:
        raise RuntimeError("no autotuning candidate ran")
    best = min(ok, key=lambda r: r["s_per_iter"])
    return {k: v for k, v in best.items() if k != "s_per_iter"}, table


def _kernel_timer(rows, cols, device, iters, fixed=False):
    import sw2d
    from sw2d import scenarios as S
    s = S.catchment(rows, dx=5.0, seed=1, cols=cols)
    h0 = np.full((rows, cols), 0.005)

    def timer(c):
        mode = dict(dt_mode=sw2d.DT_FIXED, dt=0.4) if fixed else dict(dt_mode=sw2d.DT_CFL, dt=1.0, cfl=0.5)
        g = sw2d.Solver(rows=rows, cols=cols, dx=5.0, dy=5.0, precision=sw2d.PREC_F32, south_open=1,
                        kernel=sw2d.KERNEL_STREAM, strip_h=c["strip_h"], variant=c["variant"],
                        steps_per_launch=c.get("steps_per_launch", 1 if not fixed else 0), device=device, **mode)
        try:
            g.set_static(s["z"], s["n"])
            g.set_rain(sw2d.RAIN_STEP, [50.0], 3600.0)
            g.set_state(h0)
            g.advance(6)
            g.synchronize()
            t0 = time.perf_counter()
            n = g.advance(iters)
            g.synchronize()
            return (time.perf_counter() - t0) / max(n, 1)
        finally:
            g.close()
    return timer


def tune(rows: int, cols: int, device: int = 0, cache: Optional[Cache] = None, iters: int = 48,
         strips=STRIPS, variants=VARIANTS, force: bool = False) -> dict:
    """Best (strip_h, variant) for a rows x cols grid on this GPU (cached)."""
    cache = cache or Cache()
    gpu, cls = f"{gpu_name(device)}|{TABLE_VERSION}", size_class(rows, cols)
    hit = cache.get(gpu, cls)
    if hit and not force:
        return hit
    strips = sorted(set(strips) | set(wave_strips(rows, cols, _sm_count(device))))
    cands = [{"strip_h": sh, "variant": v} for v in variants for sh in strips if sh <= max(rows, 16)]
    best, table = search(cands, _kernel_timer(rows, cols, device, iters))
    entry = {**best, "rows": rows, "cols": cols, "timings": table}
    cache.put(gpu, cls, entry)
    return entry


def fixed_candidates(rows: int, cols: int, best_one: Optional[dict] = None, variants=FIXED_VARIANTS,
                     steps=STEPS_PER_LAUNCH):
    """Candidates of tune_fixed: every build with the library's own strips
    (strip_h 0: one wave for several iterations per launch) at each number of
    iterations per launch, and the one-launch-per-iteration choice of tune()."""
    cands = [{"strip_h": 0, "variant": v, "steps_per_launch": k} for v in variants for k in steps]
    if best_one:
        cands.append({"strip_h": int(best_one["strip_h"]), "variant": int(best_one["variant"]),
                      "steps_per_launch": 1})
    return cands


def tune_fixed(rows: int, cols: int, device: int = 0, cache: Optional[Cache] = None, iters: int = 96,
               variants=FIXED_VARIANTS, steps=STEPS_PER_LAUNCH, force: bool = False) -> dict:
    """Best (strip_h, variant, steps_per_launch) under the fixed time step
    for a rows x cols grid on this GPU (cached under fixed_class)."""
    cache = cache or Cache()
    gpu = f"{gpu_name(device)}|{TABLE_VERSION}"
    hit = cache.get(gpu, fixed_class(rows, cols))
    if hit and not force:
        return hit
    one = cache.get(gpu, size_class(rows, cols))
    best, table = search(fixed_candidates(rows, cols, one, variants, steps),
                         _kernel_timer(rows, cols, device, iters, fixed=True))
    entry = {**best, "rows": rows, "cols": cols, "timings": table}
    cache.put(gpu, fixed_class(rows, cols), entry)
    return entry


def apply(cfg, cache: Optional[Cache] = None, device: int = 0):
    """Fills cfg.strip_h / cfg.variant from the cache (FP32 only), and under
    the fixed time step cfg.steps_per_launch when tune_fixed has run for the
    size class (its entry wins there); returns cfg."""
    import sw2d
    if cfg.precision != sw2d.PREC_F32:
        return cfg
    c = cache or Cache()
    gpu = f"{gpu_name(device)}|{TABLE_VERSION}"
    hit = c.get(gpu, size_class(cfg.rows, cfg.cols))
    if cfg.dt_mode == sw2d.DT_FIXED:
        fixed = c.get(gpu, fixed_class(cfg.rows, cfg.cols))
        if fixed:
            cfg.strip_h = int(fixed["strip_h"])
            cfg.variant = int(fixed["variant"])
            if cfg.steps_per_launch == 0:
                cfg.steps_per_launch = int(fixed["steps_per_launch"])
            return cfg
    if hit:
        cfg.strip_h = int(hit["strip_h"])
        cfg.variant = int(hit["variant"])
    return cfg


def _batch_timer(device, count, launches):
    import sw2d
    from sw2d import scenarios as S
    bank = S.TerrainBank(size=1024, dx=5.0, seed=3)
    ens = S.ensemble(bank, count=count, sides=(128, 256, 512, 1024), seed=4)

    def timer(c):
        b = sw2d.Batch(sw2d.batch_config(device=device, chunk=c["chunk"], variant=c["variant"],
                                         strip_h=c.get("strip_h", 0), max_scenarios=count + 1))
        try:
            for e in ens:
                cfg = sw2d.default_config(rows=e["side"], cols=e["side"], dx=5.0, dy=5.0, precision=sw2d.PREC_F32,
                                          dt_mode=sw2d.DT_CFL, dt=1.0, cfl=0.5, south_open=1, device=device)
                b.add(cfg, e["z"], np.full((e["side"], e["side"]), 0.005), manning=e["n"],
                      rain_kind=sw2d.RAIN_LINEAR, rain=e["rain"], rain_dt=e["rain_dt"], t_end=1e9)
            n = max(launches, c["chunk"])
            b.advance(c["chunk"])
            b.advance(c["chunk"] * 2)  # warm-up, including the graph builds
            t0 = time.perf_counter()
            b.advance(n)
            return (time.perf_counter() - t0) / n
        finally:
            b.close()
    return timer


def tune_batch(device: int = 0, cache: Optional[Cache] = None, variants=BATCH_VARIANTS, chunks=(12, 24, 48),
               strips=BATCH_STRIPS, count: int = 24, launches: int = 96, force: bool = False) -> dict:
    """Best (batched-kernel build, graph chunk), then the best strip height
    for that pair, on a small wet ensemble (cached)."""
    cache = cache or Cache()
    gpu = f"{gpu_name(device)}|{TABLE_VERSION}"
    hit = cache.get(gpu, BATCH_CLASS)
    if hit and not force:
        return hit
    timer = _batch_timer(device, count, launches)
    cands = [{"variant": v, "chunk": ch, "strip_h": 0} for v in variants for ch in chunks]
    best, table = search(cands, timer)
    others = [sh for sh in strips if sh != 0]
    if others:
        pair = {"variant": best["variant"], "chunk": best["chunk"]}
        t_best = min(r["s_per_iter"] for r in table if "s_per_iter" in r)
        try:
            best2, table2 = search([{**pair, "strip_h": sh} for sh in others], timer)
        except RuntimeError:  # none of the taller strips ran: keep the size rule
            best2, table2 = None, []
        table = table + table2
        ok2 = [r["s_per_iter"] for r in table2 if "s_per_iter" in r]
        if best2 is not None and ok2 and min(ok2) < t_best:
            best = best2
    entry = {**best, "timings": table}
    cache.put(gpu, BATCH_CLASS, entry)
    return entry


def apply_batch(bcfg, cache: Optional[Cache] = None):
    """Fills bcfg.variant / bcfg.chunk (and strip_h, when the cached choice
    has one and bcfg leaves it to the library) from the cache; returns bcfg."""
    hit = (cache or Cache()).get(f"{gpu_name(bcfg.device)}|{TABLE_VERSION}", BATCH_CLASS)
    if hit:
        bcfg.variant = int(hit["variant"])
        bcfg.chunk = int(hit["chunk"])
        if bcfg.strip_h == 0:
            bcfg.strip_h = int(hit.get("strip_h", 0))
    return bcfg


def tune_chunk(batch_runner: Callable[[int], float], chunks=CHUNKS) -> dict:
    """Graph chunk (iterations between host synchronisations) for a batch:
    `batch_runner(chunk)` returns seconds per iteration for that chunk."""
    best, table = search([{"chunk": c} for c in chunks], lambda c: batch_runner(c["chunk"]))
    return {**best, "timings": table}
