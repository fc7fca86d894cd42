"""Generates tests/golden/ref_evaporation.npz: the reference's own
gpu_evaporation_calc kernel (SW2D-GPU.cu:557-587), run unmodified on a GPU
through oracle/ref_harness.py, on two series:

    peri_lake   the temperature and radiation series of the reference's
                peri_lake_model dataset (tests/golden/peri_lake_db.tar.gz),
                with its albedo and its rain interval as dtime
    sweep       temperatures from -5 to 45 C against radiation from -100 to
                1400 W/m^2 (negative values exercise the clamp to 0), two
                albedos and two intervals

Needs a GPU and the device-only reference builds in oracle/_ref (made by
`make -C oracle ref` where the reference source is mounted):

    python tests/golden/make_ref_evaporation_golden.py [out.npz]
"""
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
OUT = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden", "ref_evaporation.npz")


def series():
    import refio
    with tempfile.TemporaryDirectory() as d:
        refio.extract(os.path.join(ROOT, "tests", "golden", "peri_lake_db.tar.gz"), d)
        inp = Path(d) / "peri_lake_model" / "input"
        T, Rg, albedo = refio.read_evaporation_inputs(inp / "temperatures.txt", inp / "solar_radiation.txt")
        dtrain = refio.read_rain(inp / "rain.dat")[0]
    out = [("peri_lake", T, Rg, albedo, dtrain)]
    rng = np.random.default_rng(11)
    Ts = np.linspace(-5.0, 45.0, 201)
    Rs = rng.permutation(np.linspace(-100.0, 1400.0, 201))
    out.append(("sweep_a", Ts, Rs, 0.1, 60.0))
    out.append(("sweep_b", Ts, Rs, 0.3, 3600.0))
    return out


def main():
    import ref_harness as R
    store = {}
    names = []
    for name, T, Rg, albedo, dtime in series():
        names.append(name)
        store[f"{name}__T"] = T
        store[f"{name}__Rg"] = Rg
        store[f"{name}__albedo"] = np.float64(albedo)
        store[f"{name}__dtime"] = np.float64(dtime)
        for kind in ("off", "on"):
            store[f"{name}__{kind}"] = R.evaporation(R.RefModule(kind), albedo, T, Rg, dtime)
        print(name, T.size, float(store[f"{name}__off"].max()), flush=True)
    store["cases"] = np.array(names)
    np.savez_compressed(OUT, **store)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
