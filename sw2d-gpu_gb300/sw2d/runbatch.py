"""Runs a seeded ensemble of FP32 scenarios through the batched solver and
prints its throughput.

A quick performance check of the batched path, and the command the batched
kernel's ncu summary under profiles/ was made with:

    python sw2d-gpu_gb300/sw2d/runbatch.py --count 32 --iters 96

The ensemble is the batched configuration's (scenarios.ensemble: sides
uniform over 128, 256, 512 and 1024 cells, 5 m cells cropped from one seeded
terrain, triangular hyetographs, Manning scaling, CFL 0.5, open south edge),
`--count` scenarios of it.  48 warm-up iterations, then `--iters`
iterations of every scenario, host-timed with the stream synchronised on
both sides; the throughput counts the cells of the scenarios still running.
"""
import argparse
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import sw2d  # noqa: E402
from sw2d import scenarios as S  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=32)
    ap.add_argument("--sides", type=int, nargs="+", default=[128, 256, 512, 1024])
    ap.add_argument("--iters", type=int, default=96)
    ap.add_argument("--variant", type=int, default=-1, help="-1: the library's (or the autotuner's) choice")
    ap.add_argument("--chunk", type=int, default=0, help="graph length; 0: the library's choice")
    ap.add_argument("--strip-h", type=int, default=0, help="rows per warp for every scenario; 0: by scenario size")
    ap.add_argument("--seed", type=int, default=1)
    a = ap.parse_args()
    bank = S.TerrainBank(size=max(2048, max(a.sides)), dx=5.0, seed=a.seed)
    ens = S.ensemble(bank, count=a.count, sides=tuple(a.sides), seed=a.seed + 1)
    kw = {}
    if a.variant >= 0:
        kw["variant"] = a.variant
    if a.chunk > 0:
        kw["chunk"] = a.chunk
    if a.strip_h > 0:
        kw["strip_h"] = a.strip_h
    with sw2d.Batch(device=0, max_scenarios=a.count, **kw) as b:
        ids = []
        for e in ens:
            cfg = sw2d.default_config(rows=e["side"], cols=e["side"], dx=5.0, dy=5.0, precision=sw2d.PREC_F32,
                                      dt_mode=sw2d.DT_CFL, dt=1.0, cfl=0.5, south_open=1)
            ids.append(b.add(cfg, e["z"], e["h0"], manning=e["n"], rain_kind=sw2d.RAIN_LINEAR, rain=e["rain"],
                             rain_dt=e["rain_dt"], t_end=e["t_end"]))
        b.advance(48)
        st0 = b.poll()
        t0 = time.perf_counter()
        b.advance(a.iters)  # waits for the stream
        el = time.perf_counter() - t0
        st1 = b.poll()
        cu = sum(e["side"] ** 2 * (st1[i]["steps"] - st0[i]["steps"]) for i, e in zip(ids, ens))
        print(f"scenarios={a.count} iters={a.iters} launches={b.launch_count()} {el * 1e3:.1f} ms "
              f"{cu / el:.3e} cell-updates/s (host timed)")


if __name__ == "__main__":
    main()
