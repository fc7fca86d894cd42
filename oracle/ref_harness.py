"""Runs the reference's own CUDA kernels on a GPU (TEST INFRASTRUCTURE ONLY).

oracle/_ref/sw2d_ref_fmad{off,on}.fatbin are device-only builds of the
unmodified reference source SW2D-GPU_linux/src/SW2D-GPU.cu for sm_103a, made
by `make -C oracle ref` where the reference is mounted ("off": --fmad=false,
the oracle's arithmetic; "on": nvcc's default contraction, as shipped).
This module loads them with the CUDA driver API and replays the launch
sequence of the reference's main loop (cu:1238-1241 init, cu:1256-1336 per
iteration) on zero-filled buffers of N + 2*cols elements, so the reads past
N = rows*cols + cols/2 that the reference makes in its last row (cu:654,
cu:172-174, cu:298) see zeros instead of foreign memory.

The host-side forcing of the loop (stream_flow, cu:526-555) is evaluated in
Python floats (IEEE double, the same operation order).  Kernel arguments
follow the reference signatures one to one.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FATBIN = {"off": os.path.join(HERE, "_ref", "sw2d_ref_fmadoff.fatbin"),
          "on": os.path.join(HERE, "_ref", "sw2d_ref_fmadon.fatbin")}

KERNELS = ("init_inf", "initiald", "flux", "hm_hn", "uu1_vv1", "uu_vv", "uua_vva", "continuity", "forward",
           "treat_error", "gpu_evaporation_calc")


def available(kind="off"):
    return os.path.exists(FATBIN[kind])


class _Driver:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")

    def check(self, rc, what):
        if rc != 0:
            s = C.c_char_p()
            self.cu.cuGetErrorString(rc, C.byref(s))
            raise RuntimeError(f"{what} failed: {rc} {s.value}")


class RefModule:
    """The reference kernels of one fatbin, loaded into torch's context."""

    def __init__(self, kind="off"):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.torch = torch
        self.d = _Driver()
        cu = self.d.cu
        data = open(FATBIN[kind], "rb").read()
        self._img = C.create_string_buffer(data, len(data))
        self.mod = C.c_void_p()
        self.d.check(cu.cuModuleLoadData(C.byref(self.mod), self._img), "cuModuleLoadData")
        n = C.c_uint()
        self.d.check(cu.cuModuleGetFunctionCount(C.byref(n), self.mod), "cuModuleGetFunctionCount")
        funcs = (C.c_void_p * n.value)()
        self.d.check(cu.cuModuleEnumerateFunctions(funcs, n, self.mod), "cuModuleEnumerateFunctions")
        self.fn = {}
        for f in funcs:
            name = C.c_char_p()
            self.d.check(cu.cuFuncGetName(C.byref(name), C.c_void_p(f)), "cuFuncGetName")
            nm = name.value.decode()
            for k in KERNELS:
                if nm.startswith(f"_Z{len(k)}{k}"):
                    self.fn[k] = C.c_void_p(f)
        missing = [k for k in KERNELS if k not in self.fn]
        if missing:
            raise RuntimeError(f"reference kernels not found in {FATBIN[kind]}: {missing}")

    def launch(self, name, N, *args):
        """Launches with the reference's shape: ceil(N/1024) blocks of 1024
        threads (cu:1222-1235), on the legacy default stream, then syncs."""
        vals = []
        for kind, v in args:
            if kind == "i":
                vals.append(C.c_int(int(v)))
            elif kind == "d":
                vals.append(C.c_double(float(v)))
            else:
                vals.append(C.c_void_p(int(v)))
        ptrs = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        tpb = 1024 if N >= 1024 else N
        nb = (N + tpb - 1) // tpb
        cu = self.d.cu
        self.d.check(cu.cuLaunchKernel(self.fn[name], nb, 1, 1, tpb, 1, 1, 0, None, ptrs, None), name)
        self.d.check(cu.cuCtxSynchronize(), name + " sync")


def _round_c(x):
    """C round(): half away from zero."""
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


class RefRun:
    """One case on the reference kernels (FP64), mirroring main() of the
    reference from the buffer setup (cu:1105-1213) through the loop."""

    def __init__(self, mod: RefModule, rows, cols, dx, z, h0, manning, nodata=-9999.0, dt=0.04, INT=0.0,
                 INF=0.0, LWL=0.0, EV_WL_min=0.0, rain=None, dtrain=60.0, sources=(), q=None, dtoq=60.0,
                 evapo=None):
        t = mod.torch
        self.m, self.rows, self.cols = mod, rows, cols
        self.N = rows * cols + cols // 2  # cu:829
        self.dx = self.dy = float(dx)
        self.dt, self.dt2, self.gg = float(dt), 2.00 * float(dt), 9.80  # cu:808-809
        self.rn = float(manning)
        self.INT, self.INF, self.LWL, self.EV = float(INT), float(INF), float(LWL), float(EV_WL_min)
        self.nodata = float(nodata)
        L = self.N + 2 * cols
        dev = "cuda"
        f64 = lambda: t.zeros(L, dtype=t.float64, device=dev)
        i32 = lambda: t.zeros(L, dtype=t.int32, device=dev)
        self.b = {k: f64() for k in ("baseo", "h", "um", "hm", "uu1", "umo", "vv1", "vva", "vn", "hn", "vno",
                                     "uua", "ho", "uu", "vv", "ql")}
        self.b.update({k: i32() for k in ("inf", "infx", "infy")})
        self.rr = t.zeros(1, dtype=t.float64, device=dev)
        self.Ev = t.zeros(1, dtype=t.float64, device=dev)
        self.th = t.full((1,), 1.0e-4, dtype=t.float64, device=dev)  # cu:1130
        n = rows * cols
        self.b["baseo"][:n] = t.from_numpy(np.ascontiguousarray(z, dtype=np.float64).ravel()).to(dev)
        self.b["h"][:n] = t.from_numpy(np.ascontiguousarray(h0, dtype=np.float64).ravel()).to(dev)
        self.rain = None if rain is None else [float(v) for v in rain]
        self.dtrain = float(dtrain)
        self.sources = list(sources)  # linear indices into the reference's N-vector
        self.q = None if q is None else np.asarray(q, dtype=np.float64).reshape(-1, max(1, len(self.sources)))
        self.dtoq = float(dtoq)
        self.evapo = None if evapo is None else [float(v) for v in evapo]
        self.h_ql = np.zeros(self.N, dtype=np.float64)
        self.time = 0.0
        self.steps = 0
        P = lambda k: ("p", self.b[k].data_ptr())
        N = self.N
        mod.launch("init_inf", N, ("i", rows), ("i", cols), P("ho"), P("h"), P("inf"), P("baseo"), ("i", N),
                   ("d", self.nodata))
        mod.launch("initiald", N, ("i", rows), ("i", cols), P("h"), P("infx"), P("infy"), P("inf"), P("hm"),
                   P("hn"), P("baseo"), ("i", N), ("d", self.nodata))

    # stream_flow (cu:526-555), host side
    def _stream_flow(self, time):
        for i, cell in enumerate(self.sources):
            if time <= 1.00:
                ql = self.q[0][i] * time
            else:
                it = int(time / self.dtoq)
                ql = self.q[it][i] + (self.q[it + 1][i] - self.q[it][i]) / (self.dtoq * (time - self.dtoq * (it)))
            ql = ql / (self.dx * self.dy)
            self.h_ql[cell] = ql
        if self.rain is None:
            rr = 0.0
        elif time <= 1.00:
            rr = self.rain[0] * time
        else:
            it = int(time / self.dtrain)
            try:
                rr = self.rain[it] + (self.rain[it + 1] - self.rain[it]) / (self.dtrain * (time - self.dtrain * (it)))
            except ZeroDivisionError:  # C gives x/0 = +-inf or 0/0 = NaN here
                num = self.rain[it + 1] - self.rain[it]
                rr = self.rain[it] + (math.copysign(math.inf, num) if num != 0 else math.nan)
        rr = rr / (self.dtrain * 1000.0)
        t = self.m.torch
        self.b["ql"][: self.N] = t.from_numpy(self.h_ql).to("cuda")
        self.rr.fill_(rr)
        if self.evapo is not None:  # evaporation_load, cu:589-601
            if time <= 1.00:
                ev = self.evapo[0] * time
            else:
                it = int(time / self.dtrain)
                ev = self.evapo[it] + (self.evapo[it + 1] - self.evapo[it]) / (self.dtrain * (time - self.dtrain * (it)))
            self.Ev.fill_(ev / (self.dtrain * 1000.0))

    def step(self):
        m, N, rows, cols = self.m, self.N, self.rows, self.cols
        P = lambda k: ("p", self.b[k].data_ptr())
        th, rr, Ev = ("p", self.th.data_ptr()), ("p", self.rr.data_ptr()), ("p", self.Ev.data_ptr())
        m.launch("flux", N, th, ("d", self.gg), ("d", self.rn), P("inf"), P("h"), P("infx"), P("infy"), P("baseo"),
                 P("um"), P("hm"), P("uu1"), P("umo"), P("vv1"), P("vva"), P("vn"), P("hn"), P("vno"), P("uua"),
                 P("ho"), ("i", N), ("i", cols), ("i", rows), ("d", self.dx), ("d", self.dy), ("d", self.dt2))
        cont = lambda: m.launch("continuity", N, ("d", self.dt2), ("i", cols), ("i", rows), ("d", self.dx),
                                ("d", self.dy), rr, Ev, P("ql"), P("h"), P("ho"), P("um"), P("vn"), ("d", self.INT),
                                ("d", self.INF), ("d", self.LWL), ("d", self.EV), P("inf"), ("i", N))
        self._stream_flow(self.time)
        cont()
        m.launch("treat_error", N, ("i", cols), ("i", rows), th, P("inf"), P("um"), P("vn"), P("h"), ("i", N))
        self.time = self.time + self.dt
        self._stream_flow(self.time)
        cont()
        m.launch("hm_hn", N, P("hm"), P("hn"), P("h"), ("i", N), ("i", cols), ("i", rows))
        m.launch("uu1_vv1", N, th, P("hm"), P("hn"), P("uu1"), P("um"), P("vv1"), P("vn"), ("i", N), ("i", cols),
                 ("i", rows))
        m.launch("uu_vv", N, th, P("h"), P("uu1"), P("vv1"), P("uu"), P("vv"), ("i", N), ("i", cols))
        m.launch("uua_vva", N, P("uu1"), P("vv1"), P("uua"), P("vva"), ("i", N), ("i", cols), ("i", rows))
        m.launch("forward", N, ("i", cols), ("i", rows), P("umo"), P("um"), P("vno"), P("vn"), P("ho"), P("h"),
                 ("i", N))
        self.time = self.time + self.dt
        self.steps += 1

    def run(self, nsteps):
        for _ in range(nsteps):
            self.step()

    def fields(self):
        """h (rows x cols), um ((rows+1) x cols, south wall row = 0 as read
        through the zero padding), vn (rows x (cols+1), east wall = 0),
        uu, vv (rows x cols)."""
        r, c = self.rows, self.cols
        g = lambda k: self.b[k].cpu().numpy()
        n = r * c
        h = g("h")[:n].reshape(r, c)
        um = np.zeros((r + 1, c))
        um[:r] = g("um")[:n].reshape(r, c)
        vn = np.zeros((r, c + 1))
        vn[:, :c] = g("vn")[:n].reshape(r, c)
        return {"h": h, "um": um, "vn": vn, "uu": g("uu")[:n].reshape(r, c), "vv": g("vv")[:n].reshape(r, c),
                "t": self.time, "steps": self.steps}


def evaporation(mod: RefModule, albedo, temperature, radiation, dtime):
    """The reference's gpu_evaporation_calc (cu:557-587) over a series, with
    its launch shape; returns d_Evapo [mm per record interval]."""
    t = mod.torch
    T = t.from_numpy(np.ascontiguousarray(temperature, dtype=np.float64)).to("cuda")
    Rg = t.from_numpy(np.ascontiguousarray(radiation, dtype=np.float64)).to("cuda")
    n = T.numel()
    Rs, pw, lv, ev = (t.zeros(n, dtype=t.float64, device="cuda") for _ in range(4))
    P = lambda a: ("p", a.data_ptr())
    mod.launch("gpu_evaporation_calc", n, ("d", albedo), P(T), P(Rg), P(Rs), P(pw), P(lv), P(ev), ("d", dtime),
               ("i", n))
    return ev.cpu().numpy()


def reference_cell(rows, cols, qinx, qiny):
    """The reference's linear index for a point source at cell coordinates
    (qinx, qiny) counted from the lower-left corner (cu:542-545, Linux)."""
    return (qiny + 1) * cols - (cols - (qinx + 1))
