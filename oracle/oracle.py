"""ctypes front end of the CPU oracle (oracle/sw2d_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg, where it is the checker or the timed CPU
baseline.  The product library never imports it.

Array conventions (all float64, C order, north row first):
  h, z, n   : rows x cols cells
  um        : (rows+1) x cols   x-faces, um[i, j] between cells (i-1, j) and (i, j)
  vn        : rows x (cols+1)   y-faces, vn[i, j] between cells (i, j-1) and (i, j)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

RAIN_NONE, RAIN_COMPAT, RAIN_STEP, RAIN_LINEAR, RAIN_STORM = 0, 1, 2, 3, 4


class Params(C.Structure):
    _fields_ = [
        ("rows", C.c_int32), ("cols", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double),
        ("g", C.c_double), ("th", C.c_double), ("manning", C.c_double),
        ("INT", C.c_double), ("INF", C.c_double), ("LWL", C.c_double), ("EV_WL_min", C.c_double),
        ("dt_mode", C.c_int32), ("dt", C.c_double), ("cfl", C.c_double),
        ("south_open", C.c_int32), ("pad0", C.c_int32),
    ]


class Forcing(C.Structure):
    _fields_ = [
        ("rain_kind", C.c_int32), ("n_rain", C.c_int32),
        ("rain", C.POINTER(C.c_double)), ("rain_dt", C.c_double),
        ("storm_peak", C.c_double), ("storm_x0", C.c_double), ("storm_y0", C.c_double),
        ("storm_vx", C.c_double), ("storm_vy", C.c_double), ("storm_sigma", C.c_double),
        ("storm_tstop", C.c_double),
        ("n_ev", C.c_int32), ("pad0", C.c_int32),
        ("ev", C.POINTER(C.c_double)), ("ev_dt", C.c_double),
        ("n_src", C.c_int32), ("n_qrec", C.c_int32),
        ("src_cell", C.POINTER(C.c_int32)), ("src_q", C.POINTER(C.c_double)),
        ("dtoq", C.c_double),
        ("rain_w", C.POINTER(C.c_double)),
    ]


class Budget(C.Structure):
    _fields_ = [(k, C.c_double) for k in
                ("rain_in", "source_in", "evap_out", "outflow", "clamp_gain", "cmax")]


_lib = None


def build() -> str:
    """Compile the oracle with its committed Makefile (gcc, no FMA contraction)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(Params), C.c_void_p, C.c_void_p, C.c_double]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
        L.orc_advance.restype = C.c_int64
        L.orc_advance.argtypes = [C.c_void_p, C.POINTER(Forcing), C.c_int64, C.c_double]
        L.orc_get.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.POINTER(C.c_double), C.POINTER(C.c_int64)]
        L.orc_cell_velocity.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_volume.restype = C.c_double
        L.orc_volume.argtypes = [C.c_void_p]
        L.orc_budget_get.argtypes = [C.c_void_p, C.POINTER(Budget)]
        L.orc_next_dt.restype = C.c_double
        L.orc_next_dt.argtypes = [C.c_void_p, C.c_double]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class OracleForcing:
    """Holds the numpy buffers behind a ``Forcing`` struct."""

    def __init__(self, rain_kind=RAIN_NONE, rain=None, rain_dt=1.0, storm=None,
                 ev=None, ev_dt=1.0, sources=None, src_q=None, dtoq=1.0, rain_w=None):
        self._keep = []
        f = Forcing()
        f.rain_kind = rain_kind
        if rain is not None:
            r = _f64(np.atleast_1d(rain))
            self._keep.append(r)
            f.rain = r.ctypes.data_as(C.POINTER(C.c_double))
            f.n_rain = r.size
        f.rain_dt = rain_dt
        if storm is not None:
            f.storm_peak = storm["peak"]
            f.storm_x0, f.storm_y0 = storm["x0"], storm["y0"]
            f.storm_vx, f.storm_vy = storm["vx"], storm["vy"]
            f.storm_sigma = storm["sigma"]
            f.storm_tstop = storm.get("tstop", 1e300)
        if ev is not None:
            e = _f64(np.atleast_1d(ev))
            self._keep.append(e)
            f.ev = e.ctypes.data_as(C.POINTER(C.c_double))
            f.n_ev = e.size
        f.ev_dt = ev_dt
        if sources is not None and len(sources):
            cells = np.ascontiguousarray(sources, dtype=np.int32)
            q = _f64(np.asarray(src_q).reshape(-1, cells.size))
            self._keep += [cells, q]
            f.n_src = cells.size
            f.n_qrec = q.shape[0]
            f.src_cell = cells.ctypes.data_as(C.POINTER(C.c_int32))
            f.src_q = q.ctypes.data_as(C.POINTER(C.c_double))
        f.dtoq = dtoq
        if rain_w is not None:
            w = _f64(rain_w)
            self._keep.append(w)
            f.rain_w = w.ctypes.data_as(C.POINTER(C.c_double))
        self.struct = f


class Oracle:
    """One scenario advanced by the CPU oracle."""

    def __init__(self, rows, cols, dx, dy, z, n=None, nodata=-9999.0, manning=0.0,
                 g=9.80, th=1.0e-4, INT=0.0, INF=0.0, LWL=0.0, EV_WL_min=0.0,
                 dt_mode=1, dt=0.5, cfl=0.5, south_open=0, threads=None):
        self.rows, self.cols = rows, cols
        p = Params(rows=rows, cols=cols, dx=dx, dy=dy, g=g, th=th, manning=manning,
                   INT=INT, INF=INF, LWL=LWL, EV_WL_min=EV_WL_min, dt_mode=dt_mode,
                   dt=dt, cfl=cfl, south_open=south_open)
        self.params = p
        L = lib()
        if threads is not None:
            L.orc_set_threads(int(threads))
        z = _f64(z).reshape(rows, cols)
        n = _f64(n)
        self._h = L.orc_create(C.byref(p), _ptr(z), _ptr(n), float(nodata))
        self.forcing = OracleForcing()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_destroy(h)
            self._h = None

    def set_state(self, h, um=None, vn=None, t=0.0):
        h = _f64(h)
        um, vn = _f64(um), _f64(vn)
        lib().orc_set_state(self._h, _ptr(h), _ptr(um), _ptr(vn), float(t))

    def set_forcing(self, forcing: OracleForcing):
        self.forcing = forcing

    def advance(self, max_steps, t_end=1e300):
        return int(lib().orc_advance(self._h, C.byref(self.forcing.struct), int(max_steps), float(t_end)))

    def state(self):
        r, c = self.rows, self.cols
        h = np.empty((r, c)); um = np.empty((r + 1, c)); vn = np.empty((r, c + 1))
        t = C.c_double(); s = C.c_int64()
        lib().orc_get(self._h, _ptr(h), _ptr(um), _ptr(vn), C.byref(t), C.byref(s))
        return {"h": h, "um": um, "vn": vn, "t": t.value, "steps": s.value}

    def cell_velocity(self):
        uu = np.empty((self.rows, self.cols)); vv = np.empty((self.rows, self.cols))
        lib().orc_cell_velocity(self._h, _ptr(uu), _ptr(vv))
        return uu, vv

    def volume(self):
        return float(lib().orc_volume(self._h))

    def budget(self):
        b = Budget()
        lib().orc_budget_get(self._h, C.byref(b))
        return {k: getattr(b, k) for k, _ in Budget._fields_}

    def next_dt(self, t_end=1e300):
        return float(lib().orc_next_dt(self._h, float(t_end)))


def evaporation_series(temperature, radiation, albedo, dtime):
    """The reference's evaporation per record [mm per record interval],
    restated from gpu_evaporation_calc (SW2D-GPU.cu:557-587) in numpy float64
    with the same operations in the same order: net radiation (1 - albedo)*Rg,
    the ITS-90 water density polynomial, the latent heat of Henderson-Sellers
    (1984), (Rs / (lv * pw)) * dtime * 1000, and 0 for negative values."""
    T = np.asarray(temperature, dtype=np.float64)
    Rg = np.asarray(radiation, dtype=np.float64)
    Rs = (1 - albedo) * Rg
    pw = (999.85308 + 6.32693 * (0.01) * T - 8.523829 * (0.001) * T * T + 6.943248 * (0.00001) * T * T * T
          - 3.821216 * (0.0000001) * T * T * T * T)
    a = T + 273.15
    lv = ((a / (a - 33.91)) * (a / (a - 33.91))) * 1.91846 * 1000000
    e = (Rs / (lv * pw)) * dtime * 1000.0
    return np.where(e < 0, 0.0, e)


def max_threads():
    return int(lib().orc_max_threads())
