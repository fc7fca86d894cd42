"""ctypes binding of the C ABI (include/sw2d.h) exported by libsw2d.so.

This is the Python face of the drop-in boundary: every call goes straight to
the native library; there is no Python or CPU fallback.  If the library is
missing, loading fails with an error.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libsw2d.so")
HEADER = os.path.join(os.path.dirname(PKG_ROOT), "include", "sw2d.h")

OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_NONFINITE, ERR_TIMEOUT, ERR_STATE = range(7)
PREC_F64, PREC_F32 = 0, 1
DT_FIXED, DT_CFL = 0, 1
FIELD_DEPTH, FIELD_UM, FIELD_VN, FIELD_UU, FIELD_VV, FIELD_ELEVATION = range(6)
RAIN_NONE, RAIN_COMPAT, RAIN_STEP, RAIN_LINEAR, RAIN_STORM = range(5)
KERNEL_AUTO, KERNEL_TILE, KERNEL_STREAM = range(3)


class Config(C.Structure):
    _fields_ = [
        ("rows", C.c_int32), ("cols", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("nodata", C.c_double),
        ("g", C.c_double), ("th", C.c_double), ("manning", C.c_double),
        ("INT", C.c_double), ("INF", C.c_double), ("LWL", C.c_double), ("EV_WL_min", C.c_double),
        ("precision", C.c_int32), ("dt_mode", C.c_int32),
        ("dt", C.c_double), ("cfl", C.c_double),
        ("south_open", C.c_int32), ("device", C.c_int32),
        ("tile_h", C.c_int32), ("tile_w", C.c_int32),
        ("kernel", C.c_int32), ("strip_h", C.c_int32),
        ("variant", C.c_int32), ("steps_per_launch", C.c_int32),
    ]


class Budget(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double), ("cmax", C.c_double),
        ("volume", C.c_double), ("volume0", C.c_double),
        ("rain_in", C.c_double), ("source_in", C.c_double), ("evap_out", C.c_double),
        ("outflow", C.c_double), ("clamp_gain", C.c_double),
        ("steps", C.c_int64), ("nonfinite", C.c_int32), ("reserved", C.c_int32),
    ]


class BatchConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int32), ("max_scenarios", C.c_int32), ("max_units", C.c_int32), ("strip_h", C.c_int32),
        ("max_bytes", C.c_int64), ("chunk", C.c_int32), ("variant", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("batch", BatchConfig), ("launches_per_step", C.c_int32), ("keep_depth", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]


REQ_UNKNOWN, REQ_PENDING, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = range(6)


class SW2DError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None

# every function the header declares, with its ctypes signature
_SIGS = {
    "sw2d_config_init": (C.c_int, [C.POINTER(Config)]),
    "sw2d_device_bytes": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_int64)]),
    "sw2d_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "sw2d_destroy": (C.c_int, [C.c_void_p]),
    "sw2d_set_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "sw2d_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    "sw2d_set_rain": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_double]),
    "sw2d_set_storm": (C.c_int, [C.c_void_p] + [C.c_double] * 7),
    "sw2d_set_evaporation": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_double]),
    "sw2d_evaporation_series": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_void_p]),
    "sw2d_set_point_sources": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_double]),
    "sw2d_advance": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.POINTER(C.c_int64)]),
    "sw2d_get_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "sw2d_get_budget": (C.c_int, [C.c_void_p, C.POINTER(Budget)]),
    "sw2d_probe": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "sw2d_synchronize": (C.c_int, [C.c_void_p]),
    "sw2d_get_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "sw2d_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "sw2d_describe": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32]),
    "sw2d_set_rain_weights": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sw2d_last_error": (C.c_char_p, [C.c_void_p]),
    "sw2d_status_string": (C.c_char_p, [C.c_int32]),
    "sw2d_volume_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                      C.c_void_p, C.POINTER(C.c_double)]),
    "sw2d_checkpoint_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "sw2d_checkpoint_save": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "sw2d_checkpoint_load": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "sw2d_batch_config_init": (C.c_int, [C.POINTER(BatchConfig)]),
    "sw2d_batch_scenario_bytes": (C.c_int, [C.POINTER(Config), C.c_int32, C.c_int32, C.POINTER(C.c_int64)]),
    "sw2d_batch_create": (C.c_int, [C.POINTER(BatchConfig), C.POINTER(C.c_void_p)]),
    "sw2d_batch_destroy": (C.c_int, [C.c_void_p]),
    "sw2d_batch_add": (C.c_int, [C.c_void_p, C.POINTER(Config), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                 C.c_void_p, C.c_int32, C.c_double, C.c_double, C.POINTER(C.c_int32)]),
    "sw2d_batch_advance": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]),
    "sw2d_batch_poll": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                  C.POINTER(C.c_int32)]),
    "sw2d_batch_get_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "sw2d_batch_get_budget": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(Budget)]),
    "sw2d_batch_remove": (C.c_int, [C.c_void_p, C.c_int32]),
    "sw2d_batch_bytes_in_use": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "sw2d_batch_get_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "sw2d_batch_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "sw2d_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "sw2d_server_config_init": (C.c_int, [C.POINTER(ServerConfig)]),
    "sw2d_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "sw2d_server_destroy": (C.c_int, [C.c_void_p]),
    "sw2d_server_submit": (C.c_int, [C.c_void_p, C.POINTER(Config), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                     C.c_void_p, C.c_int32, C.c_double, C.c_double, C.POINTER(C.c_int32)]),
    "sw2d_server_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "sw2d_server_poll": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                   C.POINTER(C.c_int64)]),
    "sw2d_server_get_budget": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(Budget)]),
    "sw2d_server_get_depth": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "sw2d_server_cancel": (C.c_int, [C.c_void_p, C.c_int32]),
    "sw2d_server_release": (C.c_int, [C.c_void_p, C.c_int32]),
    "sw2d_server_bytes_in_use": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "sw2d_server_get_batch": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "sw2d_server_last_error": (C.c_char_p, [C.c_void_p]),
    "sw2d_server_request_error": (C.c_char_p, [C.c_void_p, C.c_int32]),
}


def exported_names():
    return list(_SIGS)


def load(path: str | None = None):
    """Loads libsw2d.so (fails loudly when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"{p} not found: build it with sw2d-gpu_gb300/build_native.py (no CPU fallback exists)")
    L = C.CDLL(p)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


def evaporation_series(temperature, radiation, albedo, dtime):
    """The reference's energy-balance evaporation [mm per record interval] from air temperatures [deg C]
    and global radiation [W/m^2] (host computation, sw2d_evaporation_series)."""
    t = _f64(np.atleast_1d(temperature))
    r = _f64(np.atleast_1d(radiation))
    if t.shape != r.shape:
        raise ValueError("temperature and radiation series differ in length")
    out = np.empty_like(t)
    st = load().sw2d_evaporation_series(_p(t), _p(r), t.size, float(albedo), float(dtime), _p(out))
    if st != OK:
        raise SW2DError(st, "sw2d_evaporation_series")
    return out


def default_config(**kw) -> Config:
    c = Config()
    load().sw2d_config_init(C.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise AttributeError(f"sw2d_config has no field {k}")
        setattr(c, k, v)
    return c


def device_bytes(cfg: Config) -> int:
    b = C.c_int64()
    st = load().sw2d_device_bytes(C.byref(cfg), C.byref(b))
    if st != OK:
        raise SW2DError(st, "sw2d_device_bytes")
    return int(b.value)


class Solver:
    """One scenario on the GPU, owned through a C-ABI handle."""

    def __init__(self, cfg: Config | None = None, **kw):
        """Creates the handle from a Config or from its fields as keywords.  With keywords that leave the
        decomposition to the library (no strip_h, variant or kernel) an FP32 handle takes the autotuner's
        cached choice for its size class on this GPU, when there is one (sw2d.autotune)."""
        L = load()
        self.cfg = cfg if cfg is not None else default_config(**kw)
        if cfg is None and not ({"strip_h", "variant", "kernel"} & set(kw)) and self.cfg.precision == PREC_F32:
            from . import autotune
            if autotune.enabled():
                autotune.apply(self.cfg, device=self.cfg.device)
        h = C.c_void_p()
        st = L.sw2d_create(C.byref(self.cfg), C.byref(h))
        if st != OK:
            raise SW2DError(st, "sw2d_create failed: " + L.sw2d_status_string(st).decode())
        self._h = h
        self.rows, self.cols = self.cfg.rows, self.cfg.cols

    def _check(self, st, what):
        if st != OK:
            msg = load().sw2d_last_error(self._h).decode()
            raise SW2DError(st, f"{what}: {msg}")

    def close(self):
        """Frees the handle and its device memory (sw2d_destroy); safe to call twice."""
        if getattr(self, "_h", None):
            load().sw2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- inputs ---------------------------------------------------------
    def set_static(self, z, manning=None):
        """DEM z and an optional per-cell Manning raster, (rows, cols) float64, north row first; cells at
        cfg.nodata are inactive."""
        r, c = self.rows, self.cols
        z = _f64(z, (r, c))
        n = _f64(manning, (r, c)) if manning is not None else None
        self._check(load().sw2d_set_static(self._h, _p(z), _p(n)), "sw2d_set_static")

    def set_state(self, depth, um=None, vn=None, t0=0.0):
        """Depth (rows, cols) and optional discharges um (rows+1, cols) and vn (rows, cols+1) at time t0; resets
        the budgets."""
        r, c = self.rows, self.cols
        d = _f64(depth, (r, c))
        u = _f64(um, (r + 1, c)) if um is not None else None
        v = _f64(vn, (r, c + 1)) if vn is not None else None
        self._check(load().sw2d_set_state(self._h, _p(d), _p(u), _p(v), float(t0)), "sw2d_set_state")

    def set_rain(self, kind, series=None, dt_series=1.0):
        """Uniform rain: a RAIN_* kind and its series (COMPAT: the reference's formula; STEP, LINEAR: mm/h) every
        dt_series seconds."""
        s = _f64(np.atleast_1d(series)) if series is not None else None
        n = 0 if s is None else s.size
        self._check(load().sw2d_set_rain(self._h, int(kind), _p(s), n, float(dt_series)), "sw2d_set_rain")

    def set_storm(self, peak, x0, y0, vx, vy, sigma, t_stop=1e300):
        """Moving Gaussian storm cell: peak [mm/h], centre (x0 + vx t, y0 + vy t) [m], width sigma [m], until
        t_stop [s]."""
        self._check(load().sw2d_set_storm(self._h, peak, x0, y0, vx, vy, sigma, t_stop), "sw2d_set_storm")

    def set_rain_weights(self, w=None):
        """Per-cell factors of the rain rate (rows x cols), or None for uniform rain."""
        if w is None:
            self._check(load().sw2d_set_rain_weights(self._h, None), "sw2d_set_rain_weights")
            return
        w = _f64(w, (self.rows, self.cols))
        self._check(load().sw2d_set_rain_weights(self._h, _p(w)), "sw2d_set_rain_weights")

    def set_evaporation(self, series=None, dt_series=1.0):
        """Evaporation series [mm per interval] every dt_series seconds (the reference's evaporation_load),
        applied where the depth exceeds cfg.EV_WL_min."""
        s = _f64(np.atleast_1d(series)) if series is not None else None
        n = 0 if s is None else s.size
        self._check(load().sw2d_set_evaporation(self._h, _p(s), n, float(dt_series)), "sw2d_set_evaporation")

    def set_point_sources(self, cells, q, dtoq):
        """Point sources at linear cell indices with a (records, sources) table of rates [m^3/s] every dtoq
        seconds; an empty cells array removes them."""
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        q = _f64(np.asarray(q).reshape(-1, max(cells.size, 1)))
        self._check(load().sw2d_set_point_sources(self._h, _p(cells), cells.size, _p(q), q.shape[0], float(dtoq)),
                    "sw2d_set_point_sources")

    # -- running --------------------------------------------------------
    def advance(self, max_steps, t_end=1e300):
        """Advances up to max_steps iterations, stopping at t_end; returns the iterations done."""
        done = C.c_int64()
        self._check(load().sw2d_advance(self._h, int(max_steps), float(t_end), C.byref(done)), "sw2d_advance")
        return int(done.value)

    def synchronize(self):
        """Waits for the work queued on the handle's stream."""
        self._check(load().sw2d_synchronize(self._h), "sw2d_synchronize")

    def stream(self) -> int:
        """The handle's CUDA stream (a cudaStream_t as an int)."""
        s = C.c_void_p()
        self._check(load().sw2d_get_stream(self._h, C.byref(s)), "sw2d_get_stream")
        return int(s.value or 0)

    def launch_count(self) -> int:
        """Step-kernel launches issued so far."""
        n = C.c_int64()
        self._check(load().sw2d_launch_count(self._h, C.byref(n)), "sw2d_launch_count")
        return int(n.value)

    def describe(self) -> str:
        """The step kernel build and decomposition this solver runs."""
        buf = C.create_string_buffer(256)
        self._check(load().sw2d_describe(self._h, buf, 256), "sw2d_describe")
        return buf.value.decode()

    # -- outputs --------------------------------------------------------
    def field(self, which):
        """One FIELD_* raster as float64: (rows, cols), (rows+1, cols) for FIELD_UM, (rows, cols+1) for FIELD_VN."""
        r, c = self.rows, self.cols
        shape = {FIELD_UM: (r + 1, c), FIELD_VN: (r, c + 1)}.get(which, (r, c))
        out = np.empty(shape, dtype=np.float64)
        self._check(load().sw2d_get_field(self._h, int(which), _p(out)), "sw2d_get_field")
        return out

    def depth(self):
        """The depth raster (rows, cols)."""
        return self.field(FIELD_DEPTH)

    def state(self):
        """h, um and vn as float64 arrays in a dict."""
        return {"h": self.field(FIELD_DEPTH), "um": self.field(FIELD_UM), "vn": self.field(FIELD_VN)}

    def budget(self):
        """Time, iterations and the FP64 budgets (volume, rain, sources, evaporation, outflow, clamp gain) as a
        dict."""
        b = Budget()
        self._check(load().sw2d_get_budget(self._h, C.byref(b)), "sw2d_get_budget")
        return {k: getattr(b, k) for k, _ in Budget._fields_ if k != "reserved"}

    def checkpoint(self) -> bytes:
        """Bit-exact snapshot of the resident state, time, step count and budgets."""
        n = C.c_int64()
        self._check(load().sw2d_checkpoint_bytes(self._h, C.byref(n)), "sw2d_checkpoint_bytes")
        buf = C.create_string_buffer(n.value)
        self._check(load().sw2d_checkpoint_save(self._h, buf, n.value), "sw2d_checkpoint_save")
        return buf.raw

    def restore(self, ckpt: bytes):
        """Loads a checkpoint() taken from a handle of the same configuration; the run continues bit for bit."""
        self._check(load().sw2d_checkpoint_load(self._h, ckpt, len(ckpt)), "sw2d_checkpoint_load")

    def probe(self, cells):
        """Depth at linear cell indices i*cols + j; an index outside the grid raises SW2DError."""
        cells = np.ascontiguousarray(cells, dtype=np.int32)
        out = np.empty(cells.size, dtype=np.float64)
        self._check(load().sw2d_probe(self._h, _p(cells), cells.size, _p(out)), "sw2d_probe")
        return out


def batch_config(**kw) -> BatchConfig:
    c = BatchConfig()
    load().sw2d_batch_config_init(C.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise AttributeError(f"sw2d_batch_config has no field {k}")
        setattr(c, k, v)
    return c


def batch_scenario_bytes(cfg: Config, n_rain=0, with_raster=True) -> int:
    b = C.c_int64()
    st = load().sw2d_batch_scenario_bytes(C.byref(cfg), int(n_rain), int(bool(with_raster)), C.byref(b))
    if st != OK:
        raise SW2DError(st, "sw2d_batch_scenario_bytes")
    return int(b.value)


class Batch:
    """Many FP32 scenarios advanced together on one GPU (C-ABI sw2d_batch_*)."""

    def __init__(self, cfg: BatchConfig | None = None, **kw):
        """Creates the batch from a BatchConfig or from its fields as keywords.  With keywords that leave the
        kernel build and graph chunk to the library (no variant or chunk) the batch takes the autotuner's
        cached choice on this GPU, when there is one (sw2d.autotune.tune_batch)."""
        L = load()
        self.cfg = cfg if cfg is not None else batch_config(**kw)
        if cfg is None and not ({"variant", "chunk"} & set(kw)):
            from . import autotune
            if autotune.enabled():
                autotune.apply_batch(self.cfg)
        h = C.c_void_p()
        st = L.sw2d_batch_create(C.byref(self.cfg), C.byref(h))
        if st != OK:
            raise SW2DError(st, "sw2d_batch_create failed")
        self._h = h
        self.shapes = {}

    def _check(self, st, what):
        if st != OK:
            raise SW2DError(st, f"{what}: {load().sw2d_batch_last_error(self._h).decode()}")

    def close(self):
        """Frees the batch, its scenarios and their device memory; safe to call twice."""
        if getattr(self, "_h", None):
            load().sw2d_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add(self, cfg: Config, z, depth, manning=None, rain_kind=RAIN_NONE, rain=None, rain_dt=1.0, t_end=1e300):
        """Admits one FP32 CFL scenario (rasters as for Solver, a series rain kind) running to t_end; returns its
        id."""
        r, c = cfg.rows, cfg.cols
        z = _f64(z, (r, c))
        d = _f64(depth, (r, c))
        n = _f64(manning, (r, c)) if manning is not None else None
        rs = _f64(np.atleast_1d(rain)) if rain is not None else None
        sid = C.c_int32()
        self._check(load().sw2d_batch_add(self._h, C.byref(cfg), _p(z), _p(n), _p(d), int(rain_kind), _p(rs),
                                          0 if rs is None else rs.size, float(rain_dt), float(t_end), C.byref(sid)),
                    "sw2d_batch_add")
        self.shapes[sid.value] = (r, c)
        return sid.value

    def advance(self, launches, wait=True):
        """Issues `launches` iterations for every running scenario; with wait, returns how many still run."""
        run = C.c_int32()
        self._check(load().sw2d_batch_advance(self._h, int(launches), C.byref(run) if wait else None),
                    "sw2d_batch_advance")
        return run.value if wait else None

    def poll(self):
        """{id: {running, t, steps}} for every resident scenario."""
        cap = max(len(self.shapes), 1)
        ids = np.zeros(cap, np.int32); run = np.zeros(cap, np.int32); t = np.zeros(cap); steps = np.zeros(cap, np.int64)
        n = C.c_int32()
        self._check(load().sw2d_batch_poll(self._h, _p(ids), _p(run), _p(t), _p(steps), cap, C.byref(n)),
                    "sw2d_batch_poll")
        k = n.value
        return {int(i): {"running": bool(rr), "t": float(tt), "steps": int(ss)}
                for i, rr, tt, ss in zip(ids[:k], run[:k], t[:k], steps[:k])}

    def field(self, sid, which=FIELD_DEPTH):
        """One FIELD_* raster of scenario sid, shaped as Solver.field."""
        r, c = self.shapes[sid]
        shape = {FIELD_UM: (r + 1, c), FIELD_VN: (r, c + 1)}.get(which, (r, c))
        out = np.empty(shape)
        self._check(load().sw2d_batch_get_field(self._h, int(sid), int(which), _p(out)), "sw2d_batch_get_field")
        return out

    def budget(self, sid):
        """The FP64 budgets of scenario sid, as Solver.budget."""
        b = Budget()
        self._check(load().sw2d_batch_get_budget(self._h, int(sid), C.byref(b)), "sw2d_batch_get_budget")
        return {k: getattr(b, k) for k, _ in Budget._fields_ if k != "reserved"}

    def remove(self, sid):
        """Removes scenario sid and frees its memory in stream order."""
        self._check(load().sw2d_batch_remove(self._h, int(sid)), "sw2d_batch_remove")
        self.shapes.pop(sid, None)

    def bytes_in_use(self):
        """Device bytes held by the resident scenarios."""
        v = C.c_int64()
        self._check(load().sw2d_batch_bytes_in_use(self._h, C.byref(v)), "sw2d_batch_bytes_in_use")
        return int(v.value)

    def stream(self):
        """The batch's CUDA stream (a cudaStream_t as an int)."""
        s = C.c_void_p()
        self._check(load().sw2d_batch_get_stream(self._h, C.byref(s)), "sw2d_batch_get_stream")
        return int(s.value or 0)

    def launch_count(self):
        """Batch-kernel launches issued so far."""
        v = C.c_int64()
        self._check(load().sw2d_batch_launch_count(self._h, C.byref(v)), "sw2d_batch_launch_count")
        return int(v.value)


def server_config(**kw) -> ServerConfig:
    """A ServerConfig from the library's defaults; batch fields (device, max_scenarios, max_bytes, chunk,
    variant, ...) and the server's own (launches_per_step, keep_depth) as keywords."""
    c = ServerConfig()
    load().sw2d_server_config_init(C.byref(c))
    for k, v in kw.items():
        if hasattr(c.batch, k):
            setattr(c.batch, k, v)
        elif hasattr(c, k) and k != "batch":
            setattr(c, k, v)
        else:
            raise AttributeError(f"sw2d_server_config has no field {k}")
    return c


class ServerHandle:
    """The native serving loop (C-ABI sw2d_server_*): continuous batching of FP32 scenarios over one batch --
    admission in submission order by free slot and device-memory footprint, one tick per step, retirement
    with results copied to the host."""

    def __init__(self, cfg: ServerConfig | None = None, **kw):
        L = load()
        self.cfg = cfg if cfg is not None else server_config(**kw)
        h = C.c_void_p()
        st = L.sw2d_server_create(C.byref(self.cfg), C.byref(h))
        if st != OK:
            raise SW2DError(st, "sw2d_server_create failed: " + L.sw2d_status_string(st).decode())
        self._h = h
        self.shapes = {}

    def _check(self, st, what):
        if st != OK:
            raise SW2DError(st, f"{what}: {load().sw2d_server_last_error(self._h).decode()}")

    def close(self):
        """Frees the server, its batch and every resident request's device memory; safe to call twice."""
        if getattr(self, "_h", None):
            load().sw2d_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, cfg: Config, z, depth, manning=None, rain_kind=RAIN_NONE, rain=None, rain_dt=1.0, t_end=1e300):
        """Queues one FP32 CFL scenario (arguments as Batch.add); returns its request id."""
        r, c = cfg.rows, cfg.cols
        z = _f64(z, (r, c))
        d = _f64(depth, (r, c))
        n = _f64(manning, (r, c)) if manning is not None else None
        rs = _f64(np.atleast_1d(rain)) if rain is not None else None
        rid = C.c_int32()
        self._check(load().sw2d_server_submit(self._h, C.byref(cfg), _p(z), _p(n), _p(d), int(rain_kind), _p(rs),
                                              0 if rs is None else rs.size, float(rain_dt), float(t_end),
                                              C.byref(rid)), "sw2d_server_submit")
        self.shapes[rid.value] = (r, c)
        return rid.value

    def step(self):
        """One round (admit, advance, retire); returns (pending, running) after it."""
        p, r = C.c_int32(), C.c_int32()
        self._check(load().sw2d_server_step(self._h, C.byref(p), C.byref(r)), "sw2d_server_step")
        return p.value, r.value

    def poll(self, rid):
        """{state, t, steps} of request rid (state: REQ_*)."""
        st, t, n = C.c_int32(), C.c_double(), C.c_int64()
        self._check(load().sw2d_server_poll(self._h, int(rid), C.byref(st), C.byref(t), C.byref(n)),
                    "sw2d_server_poll")
        return {"state": st.value, "t": t.value, "steps": int(n.value)}

    def budget(self, rid):
        """The FP64 budgets of a finished request, as Solver.budget."""
        b = Budget()
        self._check(load().sw2d_server_get_budget(self._h, int(rid), C.byref(b)), "sw2d_server_get_budget")
        return {k: getattr(b, k) for k, _ in Budget._fields_ if k != "reserved"}

    def depth(self, rid):
        """The final depth raster of a finished request (kept with keep_depth)."""
        out = np.empty(self.shapes[rid])
        self._check(load().sw2d_server_get_depth(self._h, int(rid), _p(out)), "sw2d_server_get_depth")
        return out

    def cancel(self, rid):
        """Withdraws a pending or running request."""
        self._check(load().sw2d_server_cancel(self._h, int(rid)), "sw2d_server_cancel")

    def release(self, rid):
        """Forgets a finished, failed or cancelled request."""
        self._check(load().sw2d_server_release(self._h, int(rid)), "sw2d_server_release")
        self.shapes.pop(rid, None)

    def request_error(self, rid):
        return load().sw2d_server_request_error(self._h, int(rid)).decode()

    def bytes_in_use(self):
        v = C.c_int64()
        self._check(load().sw2d_server_bytes_in_use(self._h, C.byref(v)), "sw2d_server_bytes_in_use")
        return int(v.value)
