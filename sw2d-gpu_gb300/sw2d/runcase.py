"""Runs one synthetic catchment on the GPU and prints its throughput.

A quick performance check for users of the library, and the command the
ncu summaries under profiles/ were made with:

    python sw2d-gpu_gb300/sw2d/runcase.py --precision f32 --size 2048 --iters 6

The catchment (seeded, see scenarios.catchment) starts from a uniform 5 mm
film so that every cell does the full update; rain 50 mm/h, open south edge,
CFL 0.5 (or the reference's fixed half step with --fixed-dt, and
--steps-per-launch iterations per launch).  Three warm-up iterations, then
--iters timed iterations.
"""
import argparse
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import numpy as np  # noqa: E402

import sw2d  # noqa: E402
from sw2d import scenarios as S  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", choices=["f32", "f64"], default="f32")
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--iters", type=int, default=48)
    ap.add_argument("--kernel", type=int, default=0, help="0 auto, 1 tile, 2 stream")
    ap.add_argument("--strip-h", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0)
    ap.add_argument("--tile", type=int, nargs=2, default=(0, 0))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--fixed-dt", type=float, default=0.0,
                    help="the reference's time-step rule with this half step [s] instead of CFL 0.5")
    ap.add_argument("--steps-per-launch", type=int, default=0, help="0 = the library's choice")
    a = ap.parse_args()
    n = a.size
    prec = sw2d.PREC_F32 if a.precision == "f32" else sw2d.PREC_F64
    s = S.catchment(n, dx=5.0, seed=a.seed)
    mode = dict(dt_mode=sw2d.DT_FIXED, dt=a.fixed_dt) if a.fixed_dt > 0 else dict(dt_mode=sw2d.DT_CFL, dt=1.0,
                                                                                      cfl=0.5)
    g = sw2d.Solver(rows=n, cols=n, dx=5.0, dy=5.0, precision=prec, south_open=1, kernel=a.kernel,
                    strip_h=a.strip_h, variant=a.variant, tile_h=a.tile[0], tile_w=a.tile[1],
                    steps_per_launch=a.steps_per_launch, **mode)
    g.set_static(s["z"], s["n"])
    g.set_rain(sw2d.RAIN_STEP, [50.0], 3600.0)
    g.set_state(np.full((n, n), 0.005))
    g.advance(3)
    g.synchronize()
    t0 = time.perf_counter()
    done = g.advance(a.iters)
    g.synchronize()
    el = time.perf_counter() - t0
    print(f"precision={a.precision} size={n} kernel={a.kernel} iters={done} {el / max(done, 1) * 1e6:.1f} us/iter "
          f"{n * n * done / el:.3e} cell-updates/s (host timed); {g.describe()}")


if __name__ == "__main__":
    main()
