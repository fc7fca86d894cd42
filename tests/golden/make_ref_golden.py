"""Generates tests/golden/ref_kernels.npz: outputs of the reference's own
CUDA kernels, run unmodified on a GPU through oracle/ref_harness.py.

Needs a GPU and the device-only reference builds in oracle/_ref (made by
`make -C oracle ref` where the reference source is mounted):

    python tests/golden/make_ref_golden.py [out.npz]

Each case stores its inputs and, for both reference builds ("off" =
--fmad=false, "on" = nvcc default contraction as shipped), the final depth
and discharges.  The CPU tests replay every case through the oracle.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "sw2d-gpu_gb300"))
OUT = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden", "ref_kernels.npz")


def cases():
    from sw2d import scenarios as S
    out = []
    # 1. 1D dam break in a flat frictionless channel (walls), fixed dt
    s = S.dam_break_channel(32, 80, 1.0, x_gate=30.0)
    out.append(dict(name="channel", rows=32, cols=80, dx=1.0, z=s["z"], h0=s["h0"], manning=0.0, dt=0.02,
                    steps=300))
    # 2. the reference's own dam_break dataset with its friction (n = 0.012)
    d = np.load(os.path.join(ROOT, "tests", "golden", "dam_break.npz"))
    out.append(dict(name="dam_break", rows=100, cols=100, dx=10.0, z=d["z"], h0=d["h0"],
                    manning=float(d["manning"]), dt=float(d["dt"]), INT=float(d["INT"]), INF=float(d["INF"]),
                    LWL=float(d["LWL"]), EV_WL_min=float(d["EV_WL_min"]), steps=150))
    # 3./4. terrain with NODATA holes, the reference's rain formula (mm per
    # interval, cu:547-554), point sources incl. a sink and two sources on
    # one cell, runoff fractions; without and with friction
    rows, cols = 40, 48
    c = S.catchment(rows, dx=10.0, seed=7, cols=cols, manning=0.0)
    z = c["z"].copy()
    rng = np.random.default_rng(9)
    z[rng.random(z.shape) < 0.04] = -9999.0
    h0 = np.where((z != -9999.0) & (z < np.percentile(z[z != -9999.0], 25)), 0.3, 0.0)
    from ref_harness import reference_cell
    src = [reference_cell(rows, cols, 7, 30), reference_cell(rows, cols, 30, 10), reference_cell(rows, cols, 30, 10),
           reference_cell(rows, cols, 3, 5)]
    q = np.array([[0.5, 1.0, 2.0, -0.12], [1.5, 0.0, 3.0, -0.12], [0.2, 0.5, 1.0, -0.12], [0.0, 0.0, 0.0, -0.12],
                  [0.8, 0.3, 0.0, -0.12], [0.0, 0.0, 0.5, -0.12], [0.0, 0.0, 0.0, -0.12], [0.0, 0.0, 0.0, -0.12]])
    rain = [0.0, 3.0, 6.0, 1.0, 0.0, 2.0, 0.0, 0.0]
    for name, n in (("terrain_rain_sources", 0.0), ("terrain_rain_sources_friction", 0.03)):
        out.append(dict(name=name, rows=rows, cols=cols, dx=10.0, z=z, h0=h0, manning=n, dt=0.05, steps=200,
                        INT=0.45, INF=0.20, LWL=0.30, EV_WL_min=0.05, rain=rain, dtrain=3.71, sources=src, q=q,
                        dtoq=4.33))
    return out


def main():
    import ref_harness as R
    store = {}
    names = []
    for c in cases():
        names.append(c["name"])
        p = f"{c['name']}__"
        for k in ("rows", "cols", "dx", "z", "h0", "manning", "dt", "steps", "INT", "INF", "LWL", "EV_WL_min",
                  "rain", "dtrain", "sources", "q", "dtoq"):
            if k in c:
                store[p + k] = np.asarray(c[k])
        for kind in ("off", "on"):
            mod = R.RefModule(kind)
            kw = {k: c[k] for k in ("INT", "INF", "LWL", "EV_WL_min", "rain", "dtrain", "sources", "q", "dtoq")
                  if k in c}
            run = R.RefRun(mod, c["rows"], c["cols"], c["dx"], c["z"], c["h0"], c["manning"], dt=c["dt"], **kw)
            run.run(c["steps"])
            f = run.fields()
            store[p + f"{kind}_h"] = f["h"]
            store[p + f"{kind}_t"] = np.float64(f["t"])
            if kind == "off":
                store[p + "off_um"] = f["um"]
                store[p + "off_vn"] = f["vn"]
                store[p + "off_uu"] = f["uu"]
                store[p + "off_vv"] = f["vv"]
            print(c["name"], kind, "h range", float(f["h"].min()), float(f["h"].max()), "t", f["t"], flush=True)
    store["cases"] = np.array(names)
    np.savez_compressed(OUT, **store)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
