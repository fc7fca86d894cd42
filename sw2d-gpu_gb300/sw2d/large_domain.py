"""The large-single-domain configuration: FP32 state against the FP64 path.

A catchment DEM (as in the catchment configuration) with uniform Manning
n = 0.05, rain from a Gaussian storm cell (peak 80 mm/h, sigma 2 km) whose
centre moves at 10 m/s along the north-west -> south-east diagonal from the
north-west corner, open south edge, CFL 0.5.  The FP32 run is compared with
the FP64 run of the same scenario on the GPU at the same simulated time:
max |dh| and its distribution, flooded area (h > th), relative volume error
of the FP64 budget, and the FP32 kernel's cell-update rate and algorithmic
HBM rate.

With --sensitivity the FP32 and FP64 runs are repeated with the storm peak
raised by one part in a million, and the same statistics are reported for
each path against its own unperturbed run: the pointwise spread that the
flow itself produces from a perturbation of that size, against which the
FP32/FP64 difference is read.

    python sw2d-gpu_gb300/sw2d/large_domain.py --size 8192 --dx 2 --horizon 3600 [--sensitivity]
"""
import argparse
import json
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import numpy as np  # noqa: E402

import sw2d  # noqa: E402
from sw2d import scenarios as S  # noqa: E402

TH = 1.0e-4


def storm_params(size, dx):
    v = 10.0 / np.sqrt(2.0)  # 10 m/s along the diagonal
    return dict(peak=80.0, x0=0.0, y0=0.0, vx=v, vy=v, sigma=2000.0)


def run(precision, s, size, dx, horizon, dt_max=1.0, device=0, peak_scale=1.0):
    g = sw2d.Solver(rows=size, cols=size, dx=dx, dy=dx, precision=precision, dt_mode=sw2d.DT_CFL, dt=dt_max,
                    cfl=0.5, south_open=1, manning=0.05, device=device)
    g.set_static(s["z"])
    st = storm_params(size, dx)
    g.set_storm(st["peak"] * peak_scale, st["x0"], st["y0"], st["vx"], st["vy"], st["sigma"])
    g.set_state(s["h0"])
    g.synchronize()
    t0 = time.perf_counter()
    n = g.advance(10 ** 9, t_end=horizon)
    g.synchronize()
    el = time.perf_counter() - t0
    out = {"iterations": n, "seconds": el, "cell_updates_per_s": size * size * n / el, "budget": g.budget(),
           "depth": g.depth()}
    g.close()
    return out


def spread(a, c):
    """Pointwise statistics of |a - c| (metres) and of the wet masks."""
    d = np.abs(a - c)
    wa, wc = np.count_nonzero(a > TH), np.count_nonzero(c > TH)
    return {"max": float(d.max()), "p50": float(np.percentile(d, 50)), "p99": float(np.percentile(d, 99)),
            "p99.99": float(np.percentile(d, 99.99)), "cells_over_1mm": int(np.count_nonzero(d > 1e-3)),
            "wet_cells": int(wa), "flooded_area_rel_diff": abs(wa - wc) / max(wa, 1)}


def compare(size=8192, dx=2.0, horizon=3600.0, seed=3, with_f64=True, sensitivity=False):
    s = S.catchment(size, dx=dx, seed=seed, manning=0.05)
    r32 = run(sw2d.PREC_F32, s, size, dx, horizon)
    b = r32["budget"]
    rhs = b["volume0"] + b["rain_in"] + b["source_in"] - b["evap_out"] - b["outflow"] + b["clamp_gain"]
    res = {
        "size": size, "dx": dx, "horizon_s": horizon,
        "f32": {"iterations": r32["iterations"], "seconds": r32["seconds"],
                "cell_updates_per_s": r32["cell_updates_per_s"],
                "alg_hbm_gbs": 28.0 * r32["cell_updates_per_s"] / 1e9,  # scalar n: 28 B per cell-update
                "volume": b["volume"], "rain_in": b["rain_in"], "outflow": b["outflow"],
                "volume_rel_error": abs(b["volume"] - rhs) / max(b["volume"], 1e-30)},
    }
    if with_f64:
        r64 = run(sw2d.PREC_F64, s, size, dx, horizon)
        a, c = r64["depth"], r32["depth"]
        wa, wc = np.count_nonzero(a > TH), np.count_nonzero(c > TH)
        res["f64"] = {"iterations": r64["iterations"], "seconds": r64["seconds"],
                      "cell_updates_per_s": r64["cell_updates_per_s"]}
        res["max_abs_dh_m"] = float(np.max(np.abs(a - c)))
        res["flooded_area_rel_diff"] = abs(wa - wc) / max(wa, 1)
        res["speedup_f32_over_f64"] = r64["seconds"] / r32["seconds"]
        res["f64_vs_f32"] = spread(a, c)
        if sensitivity:
            p64 = run(sw2d.PREC_F64, s, size, dx, horizon, peak_scale=1.0 + 1e-6)["depth"]
            res["f64_vs_f64_peak_1e-6"] = spread(a, p64)
            del p64
    if sensitivity:
        p32 = run(sw2d.PREC_F32, s, size, dx, horizon, peak_scale=1.0 + 1e-6)["depth"]
        res["f32_vs_f32_peak_1e-6"] = spread(r32["depth"], p32)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=8192)
    ap.add_argument("--dx", type=float, default=2.0)
    ap.add_argument("--horizon", type=float, default=3600.0)
    ap.add_argument("--no-f64", action="store_true")
    ap.add_argument("--sensitivity", action="store_true")
    a = ap.parse_args()
    print(json.dumps(compare(a.size, a.dx, a.horizon, with_f64=not a.no_f64, sensitivity=a.sensitivity)))


if __name__ == "__main__":
    main()
