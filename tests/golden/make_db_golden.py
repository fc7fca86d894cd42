"""Builds the fixtures made from the reference's two datasets
(SW2D-GPU_linux/src/db/dam_break and db/peri_lake_model):

    dam_break.npz           the dam_break inputs (DEM, initial depth,
                            setup.dat values) and its shipped output
                            output/Results_0.vtk, the one known-answer vector
                            the reference ships: the first VTK written by its
                            solver loop (SW2D-GPU.cu:1339-1472), i.e. depth =
                            initial condition and velocities after ONE
                            iteration, stored as the floats the VTK prints
    dam_break_db.tar.gz     the dam_break input files and that VTK, byte for
                            byte, for the end-to-end test of the
                            reference-format driver
    peri_lake_db.tar.gz     the peri_lake_model input files, byte for byte
                            (the reference ships no output for it)

Run where the reference project is mounted (it is not on the GPU machine), with
its root given as the argument or in SW2D_REF_ROOT:

    python tests/golden/make_db_golden.py [REF_ROOT]
"""
import gzip
import io
import os
import sys
import tarfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "dam_break.npz")
OUT_DB = os.path.join(HERE, "dam_break_db.tar.gz")
OUT_PERI = os.path.join(HERE, "peri_lake_db.tar.gz")


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


def pack(case, name, subdirs, out):
    """The case's files under <name>/<sub>/, byte for byte, fixed mtimes (the
    archive is the same on every run)."""
    with gzip.GzipFile(out, "wb", mtime=0) as gz, tarfile.open(fileobj=gz, mode="w") as tf:
        for sub in subdirs:
            for fn in sorted(os.listdir(os.path.join(case, sub))):
                path = os.path.join(case, sub, fn)
                data = open(path, "rb").read()
                info = tarfile.TarInfo(f"{name}/{sub}/{fn}")
                info.size = len(data)
                info.mtime = 0
                tf.addfile(info, io.BytesIO(data))
    print("wrote", out, os.path.getsize(out), "bytes")


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SW2D_REF_ROOT")
    if not root:
        sys.exit("give the reference project's root as the argument or in SW2D_REF_ROOT")
    db = os.path.join(root, "SW2D-GPU_linux", "src", "db")
    if not os.path.isdir(db):
        sys.exit(f"no reference datasets under {db}")
    case = os.path.join(db, "dam_break")
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
    pack(case, "dam_break", ("input", "output"), OUT_DB)
    pack(os.path.join(db, "peri_lake_model"), "peri_lake_model", ("input",), OUT_PERI)


if __name__ == "__main__":
    main()
