"""Readers of the reference's input files, for the tests that run its
datasets (SW2D-GPU_linux/src/SW2D-GPU.cu, "cu:<line>").  They follow the
reference's own reading order, independently of the C++ driver under test.
"""
import math
import tarfile

import numpy as np


def extract(tar_path, dest):
    with tarfile.open(tar_path) as tf:
        tf.extractall(dest)


def tokens(path):
    with open(path, "rb") as f:
        return f.read().decode("latin-1").split()


def read_setup(path):
    """setup.dat: "key: values" lines (cu:779-805)."""
    vals = {}
    with open(path, "rb") as f:
        for line in f.read().decode("latin-1").splitlines():
            if ":" not in line:
                continue
            k, v = line.split(":", 1)
            vals[k.strip()] = [float(x) for x in v.split()]
    return vals


def read_esri(path):
    """ESRI ASCII grid: header pairs, then rows*cols values, north row first
    (cu:815-835).  Returns (header dict with lower-case keys, rows x cols)."""
    t = tokens(path)
    hdr, k = {}, 0
    while True:
        try:
            float(t[k])
            break
        except ValueError:
            hdr[t[k].lower()] = float(t[k + 1])
            k += 2
    rows, cols = int(hdr["nrows"]), int(hdr["ncols"])
    vals = np.array([float(x) for x in t[k:k + rows * cols]], dtype=np.float64)
    return hdr, vals.reshape(rows, cols)


def read_rain(path):
    """rain.dat: dtrain, a header of four words, then "time value" lines; the
    reference reads (newlines - 1) values and runs to (newlines - 2) * dtrain
    when setup.dat gives no end time (cu:929-960, cu:1085-1087)."""
    raw = open(path, "rb").read()
    newlines = raw.count(b"\n")
    t = raw.decode("latin-1").split()
    dtrain = float(t[0])
    values = [float(x) for x in t[6::2]]
    return dtrain, np.array(values), (newlines - 2) * dtrain


def read_coords(path):
    """coord_source_sink.dat / coord_out.dat: "nst N" or "n_out N", then N
    coordinate pairs in metres (cu:848-855, cu:1047-1069)."""
    t = tokens(path)
    n = int(t[1])
    return [(float(t[2 + 2 * i]), float(t[3 + 2 * i])) for i in range(n)]


def read_q(path, nst):
    """Q_source_sink.dat: a "flow (...)" header, then nst values per record
    (cu:878-921); returns records x nst."""
    t = tokens(path)[2:]
    v = np.array([float(x) for x in t])
    return v[: (v.size // nst) * nst].reshape(-1, nst)


def read_evaporation_inputs(temperature_path, radiation_path):
    """temperatures.txt (a header word, then deg C) and solar_radiation.txt
    ("albedo: a", a header word, then W/m^2) (cu:985-1007)."""
    T = np.array([float(x) for x in tokens(temperature_path)[1:]])
    r = tokens(radiation_path)
    albedo = float(r[1])
    Rg = np.array([float(x) for x in r[3:]])
    n = min(T.size, Rg.size)
    return T[:n], Rg[:n], albedo


def c_round(x):
    """C round(): half away from zero."""
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def source_cell(hdr, rows, cols, x, y):
    """The reference's linear cell index of a point source at (x, y) metres
    (stream_flow, cu:542-545, Linux build): row counted from the top by
    rows - round(|yll - y| / res), plus one row."""
    res = hdr["cellsize"]
    qinx = c_round(abs(hdr["xllcorner"] / res - x / res))
    qiny = rows - c_round(abs(hdr["yllcorner"] / res - y / res))
    return (qiny + 1) * cols - (cols - (qinx + 1))


def probe_cell(hdr, rows, cols, x, y):
    """The reference's linear index of a WaterLevel probe (cu:1388-1398)."""
    res = hdr["cellsize"]
    outx = c_round(abs(hdr["xllcorner"] / res - x / res))
    outy = rows - c_round(abs(hdr["yllcorner"] / res - y / res))
    return outy * cols - (cols - (outx + 1))


def read_vtk_fields(path, rows, cols):
    """The SCALARS blocks of a VTK file the driver wrote, as the strings it
    printed, flipped back to north-first order (the VTK's first row is the
    grid's last, cu:1381)."""
    lines = open(path).read().split("\n")
    out = {}
    for k, line in enumerate(lines):
        if line.startswith("SCALARS"):
            name = line.split()[1]
            vals = lines[k + 2:k + 2 + rows * cols]
            out[name] = np.array(vals, dtype=object).reshape(rows, cols)[::-1]
    return out
