"""Builds tests/golden/dam_break.npz and tests/golden/dam_break_db.tar.gz
from the reference's dam_break case.

Run here, where the reference is mounted (it is not on the GPU machine):

    python tests/golden/make_dam_break_golden.py [/path/to/SW2D-GPU_linux/src/db/dam_break]

The fixture holds the case's inputs (DEM, initial depth, setup.dat values)
and the reference's shipped output db/dam_break/output/Results_0.vtk, the one
known-answer vector the reference ships: the first VTK written by its solver
loop (SW2D-GPU.cu:1339-1472), i.e. depth = initial condition and velocities
after ONE iteration.  Values are stored as the floats the VTK prints ("%f").

dam_break_db.tar.gz holds the case's input files and that VTK byte for byte,
for the end-to-end test of the reference-format driver.
"""
import io
import os
import sys
import tarfile

import numpy as np

DEFAULT = "/root/reference/SW2D-GPU_linux/src/db/dam_break"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dam_break.npz")
OUT_DB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dam_break_db.tar.gz")


def read_setup(path):
    vals = {}
    with open(path) as f:
        for line in f:
            if ":" not in line:
                continue
            k, v = line.split(":", 1)
            vals[k.strip()] = [float(x) for x in v.split()]
    return vals


def read_esri(path):
    with open(path) as f:
        toks = f.read().split()
    hdr = {}
    k = 0
    while not _isnum(toks[k]):
        hdr[toks[k].lower()] = float(toks[k + 1])
        k += 2
    data = np.array([float(x) for x in toks[k:]], dtype=np.float64)
    return hdr, data


def _isnum(s):
    try:
        float(s)
        return True
    except ValueError:
        return False


def read_vtk(path):
    fields = {}
    with open(path) as f:
        lines = [l.strip() for l in f]
    i = 0
    while i < len(lines):
        if lines[i].startswith("SCALARS"):
            name = lines[i].split()[1]
            i += 2  # skip LOOKUP_TABLE
            vals = []
            while i < len(lines) and lines[i] and not lines[i].startswith("SCALARS"):
                vals.append(float(lines[i]))
                i += 1
            fields[name] = np.array(vals)
        else:
            i += 1
    return fields


def main():
    case = sys.argv[1] if len(sys.argv) > 1 else DEFAULT
    setup = read_setup(os.path.join(case, "input", "setup.dat"))
    hdr, dem = read_esri(os.path.join(case, "input", "dem.txt"))
    rows, cols = int(hdr["nrows"]), int(hdr["ncols"])
    with open(os.path.join(case, "input", "initial_condition.txt")) as f:
        ic = np.array([float(x) for x in f.read().split()], dtype=np.float64)
    vtk = read_vtk(os.path.join(case, "output", "Results_0.vtk"))
    np.savez_compressed(
        OUT,
        rows=rows, cols=cols, dx=hdr["cellsize"], nodata=hdr["nodata_value"],
        z=dem[: rows * cols].reshape(rows, cols),
        h0=ic[: rows * cols].reshape(rows, cols),
        dt=setup["dt"][0], manning=setup["manning_coef"][0],
        INT=setup["INT"][0], INF=setup["INF"][0], LWL=setup["LWL"][0],
        EV_WL_min=setup["EV_WL_min"][0],
        vtk_depth=vtk["depth"], vtk_x_velocity=vtk["x_velocity"],
        vtk_y_velocity=vtk["y_velocity"], vtk_elevation=vtk["Elevations"],
    )
    print("wrote", OUT, {k: v.shape for k, v in vtk.items()})
    with tarfile.open(OUT_DB, "w:gz") as tf:
        for sub in ("input", "output"):
            for fn in sorted(os.listdir(os.path.join(case, sub))):
                path = os.path.join(case, sub, fn)
                data = open(path, "rb").read()
                info = tarfile.TarInfo(f"dam_break/{sub}/{fn}")
                info.size = len(data)
                info.mtime = 0
                tf.addfile(info, io.BytesIO(data))
    print("wrote", OUT_DB, os.path.getsize(OUT_DB), "bytes")


if __name__ == "__main__":
    main()
