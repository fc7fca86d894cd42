"""Continuous batching of flood scenarios on one GPU.

Requests (a scenario: rasters, forcing, simulated horizon) arrive over time.
The server keeps every admitted scenario resident in one `Batch` and
advances all of them together, a tick of `launches_per_tick` iterations at a
time.  Between ticks it

  * admits arrived requests in arrival order while their device footprint
    fits the memory budget (a request that does not fit waits; smaller ones
    behind it may pass it, so memory freed by one retirement is used at once),
  * retires the scenarios whose plan has stopped (simulated horizon reached),
    downloading their result (depth raster and FP64 budget),
  * records per request: arrival, admission and completion times.

Nothing here touches the numerics: each scenario advances exactly as it
would alone (per-scenario clocks and CFL steps in the batched kernel).

`Server` schedules in Python over a `Batch`; its backend is injected
(`batch_factory`), so the scheduling logic is tested on the host with a fake
batch.  `NativeServer` runs the same policy through the library's own loop
(`ServerHandle`, the C ABI's sw2d_server_*) and keeps only the arrival clock
and the statistics here.
"""
from __future__ import annotations

import dataclasses
import heapq
import time
from typing import Callable, Optional

import numpy as np

from .native import SW2DError


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float                 # seconds from the start of the run
    cfg: object                    # sw2d Config (FP32, CFL)
    z: np.ndarray
    depth: np.ndarray
    manning: Optional[np.ndarray]
    rain_kind: int
    rain: Optional[np.ndarray]
    rain_dt: float
    t_end: float                   # simulated horizon [s]
    bytes: int = 0                 # device footprint in the batch
    # filled by the server
    admitted: Optional[float] = None
    finished: Optional[float] = None
    result: Optional[dict] = None


class Server:
    def __init__(self, batch_factory: Callable[[], object], bytes_of: Callable[[Request], int],
                 max_bytes: int, launches_per_tick: int = 24, keep_results=False,
                 clock: Callable[[], float] = time.perf_counter, sleep: Callable[[float], None] = time.sleep):
        self.batch = batch_factory()
        # scenario slots of the batch (0 = no limit known): a request waits for
        # a free slot as it waits for memory
        self.max_running = int(getattr(getattr(self.batch, "cfg", None), "max_scenarios", 0) or 0)
        self.bytes_of = bytes_of
        self.max_bytes = int(max_bytes)
        self.launches_per_tick = int(launches_per_tick)
        self.keep_results = keep_results
        self.clock = clock
        self.sleep = sleep
        self.pending: list = []         # heap of (arrival, rid, Request) not yet admitted
        self.running: dict = {}         # scenario id -> Request
        self.done: list = []
        self.bytes_used = 0
        self.peak_bytes = 0
        self.ticks = 0
        self.t0 = None

    # ---- submission ----------------------------------------------------------
    def submit(self, req: Request):
        req.bytes = int(self.bytes_of(req))
        if req.bytes > self.max_bytes:
            raise ValueError(f"request {req.rid} needs {req.bytes} bytes, more than the budget {self.max_bytes}")
        heapq.heappush(self.pending, (req.arrival, req.rid, req))

    def poll(self, rid):
        """State of request `rid`: "pending", "running", "done", "failed",
        "cancelled", or None if the server does not know it."""
        for _, r, _req in self.pending:
            if r == rid:
                return "pending"
        if any(req.rid == rid for req in self.running.values()):
            return "running"
        for req in self.done:
            if req.rid == rid:
                if req.result.get("cancelled"):
                    return "cancelled"
                return "failed" if "error" in req.result else "done"
        return None

    def cancel(self, rid) -> bool:
        """Withdraws request `rid`: a pending one leaves the queue, a running
        one is removed from the batch between ticks and its memory returned.
        Returns False if the request is unknown or already finished."""
        now = self.now() if self.t0 is not None else 0.0
        for k, (_, r, req) in enumerate(self.pending):
            if r == rid:
                self.pending.pop(k)
                heapq.heapify(self.pending)
                req.finished, req.result = now, {"cancelled": True}
                self.done.append(req)
                return True
        for sid, req in list(self.running.items()):
            if req.rid == rid:
                self.batch.remove(sid)
                del self.running[sid]
                self.bytes_used -= req.bytes
                req.finished, req.result = now, {"cancelled": True}
                self.done.append(req)
                return True
        return False

    # ---- one scheduling round ------------------------------------------------
    def now(self):
        return self.clock() - self.t0

    def _admit(self):
        now = self.now()
        waiting = []
        while self.pending and self.pending[0][0] <= now:
            waiting.append(heapq.heappop(self.pending))
        for item in waiting:
            req = item[2]
            slot_free = not self.max_running or len(self.running) < self.max_running
            if slot_free and self.bytes_used + req.bytes <= self.max_bytes:
                try:
                    sid = self.batch.add(req.cfg, req.z, req.depth, manning=req.manning, rain_kind=req.rain_kind,
                                         rain=req.rain, rain_dt=req.rain_dt, t_end=req.t_end)
                except (SW2DError, ValueError) as e:  # refused by the library: this request fails alone
                    req.admitted = req.finished = self.now()
                    req.result = {"error": str(e)}
                    self.done.append(req)
                    continue
                req.admitted = self.now()
                self.running[sid] = req
                self.bytes_used += req.bytes
                self.peak_bytes = max(self.peak_bytes, self.bytes_used)
            else:
                heapq.heappush(self.pending, item)  # waits for memory, keeps its place

    def _retire(self):
        status = self.batch.poll()
        for sid, st in status.items():
            if sid in self.running and not st["running"]:
                req = self.running.pop(sid)
                res = {"t": st["t"], "steps": st["steps"], "budget": self.batch.budget(sid)}
                keep = self.keep_results(req) if callable(self.keep_results) else self.keep_results
                if keep:  # True, or a predicate choosing the requests whose depth raster is kept
                    res["depth"] = self.batch.field(sid)
                req.result = res
                req.finished = self.now()
                self.batch.remove(sid)
                self.bytes_used -= req.bytes
                self.done.append(req)

    def step(self):
        """Admit, advance one tick if anything is resident, retire."""
        if self.t0 is None:  # the server's clock starts at its first step
            self.t0 = self.clock()
        self._admit()
        if self.running:
            self.batch.advance(self.launches_per_tick, wait=False)
            self.ticks += 1
            self._retire()
            return True
        return False

    def run(self, requests=(), timeout=None):
        """Serves `requests` (plus anything submitted before) until all are done."""
        for r in requests:
            self.submit(r)
        if self.t0 is None:
            self.t0 = self.clock()
        while self.pending or self.running:
            if timeout is not None and self.now() > timeout:
                raise TimeoutError(f"{len(self.pending)} pending and {len(self.running)} running after {timeout} s")
            if not self.step():
                # idle: wait for the next arrival
                nxt = self.pending[0][0] - self.now()
                if nxt > 0:
                    self.sleep(min(nxt, 0.05))
        return self.stats()

    def stats(self):
        return summarize(self.done, self.peak_bytes, self.ticks)


def summarize(done, peak_bytes, ticks):
    """p50/p99/mean time to result, scenarios/hour, cell-updates/s and peak
    bytes of a finished serving run (requests with their results)."""
    if not done:
        return {"requests": 0}
    served = [r for r in done if "error" not in r.result and not r.result.get("cancelled")]
    cancelled = sum(1 for r in done if r.result.get("cancelled"))
    if not served:
        return {"requests": 0, "failed": len(done) - cancelled, "cancelled": cancelled}
    ttr = np.array([r.finished - r.arrival for r in served])
    span = max(r.finished for r in served) - min(r.arrival for r in served)
    cu = sum(int(r.cfg.rows) * int(r.cfg.cols) * int(r.result["steps"]) for r in served)
    return {
        "requests": len(served),
        "failed": len(done) - len(served) - cancelled,
        "cancelled": cancelled,
        "p50_s": float(np.percentile(ttr, 50)),
        "p99_s": float(np.percentile(ttr, 99)),
        "mean_s": float(ttr.mean()),
        "scenarios_per_hour": len(done) / span * 3600.0 if span > 0 else None,
        "cell_updates_per_s": cu / span if span > 0 else None,
        "peak_bytes": int(peak_bytes),
        "ticks": ticks,
        "span_s": float(span),
    }


class NativeServer:
    """The same serving run through the library's own loop (sw2d_server_*,
    C++ in libsw2d): admission, advancing and retirement happen there; this
    class submits each request when its arrival time comes, records arrival
    and completion times, keeps the results asked for and computes the
    statistics.  `server_factory` returns a ServerHandle (or a stand-in with
    its methods); its keep_depth must be set when keep_results asks for
    depth rasters."""

    def __init__(self, server_factory: Callable[[], object], keep_results=False,
                 clock: Callable[[], float] = time.perf_counter, sleep: Callable[[float], None] = time.sleep):
        from .native import REQ_CANCELLED, REQ_DONE, REQ_FAILED, REQ_PENDING
        self._done_states = (REQ_DONE, REQ_FAILED, REQ_CANCELLED)
        self._REQ_DONE, self._REQ_FAILED, self._REQ_PENDING = REQ_DONE, REQ_FAILED, REQ_PENDING
        self.server = server_factory()
        self.keep_results = keep_results
        self.clock = clock
        self.sleep = sleep
        self.pending: list = []   # heap of (arrival, rid, Request) not yet arrived
        self.active: dict = {}    # native request id -> Request
        self.done: list = []
        self.peak_bytes = 0
        self.ticks = 0
        self.t0 = None

    def close(self):
        close = getattr(self.server, "close", None)
        if close:
            close()

    def submit(self, req: Request):
        heapq.heappush(self.pending, (req.arrival, req.rid, req))

    def now(self):
        return self.clock() - self.t0

    def _arrivals(self):
        while self.pending and self.pending[0][0] <= self.now():
            req = heapq.heappop(self.pending)[2]
            try:
                nid = self.server.submit(req.cfg, req.z, req.depth, manning=req.manning, rain_kind=req.rain_kind,
                                         rain=req.rain, rain_dt=req.rain_dt, t_end=req.t_end)
            except (SW2DError, ValueError) as e:  # refused (larger than the whole budget, bad arguments)
                req.admitted = req.finished = self.now()
                req.result = {"error": str(e)}
                self.done.append(req)
                continue
            self.active[nid] = req

    def step(self):
        """Submit the arrived requests, run one round of the native loop, collect the finished ones."""
        if self.t0 is None:
            self.t0 = self.clock()
        self._arrivals()
        if not self.active:
            return False
        self.server.step()
        self.ticks += 1
        self.peak_bytes = max(self.peak_bytes, int(self.server.bytes_in_use()))
        now = self.now()
        for nid, req in list(self.active.items()):
            st = self.server.poll(nid)
            if req.admitted is None and st["state"] != self._REQ_PENDING:
                req.admitted = now
            if st["state"] not in self._done_states:
                continue
            if st["state"] == self._REQ_DONE:
                res = {"t": st["t"], "steps": st["steps"], "budget": self.server.budget(nid)}
                keep = self.keep_results(req) if callable(self.keep_results) else self.keep_results
                if keep:
                    res["depth"] = self.server.depth(nid)
            elif st["state"] == self._REQ_FAILED:
                res = {"error": self.server.request_error(nid)}
            else:
                res = {"cancelled": True}
            req.result, req.finished = res, now
            self.server.release(nid)
            del self.active[nid]
            self.done.append(req)
        return True

    def run(self, requests=(), timeout=None):
        """Serves `requests` (plus anything submitted before) until all are done."""
        for r in requests:
            self.submit(r)
        if self.t0 is None:
            self.t0 = self.clock()
        while self.pending or self.active:
            if timeout is not None and self.now() > timeout:
                raise TimeoutError(f"{len(self.pending)} waiting to arrive and {len(self.active)} in the server "
                                   f"after {timeout} s")
            if not self.step():
                nxt = self.pending[0][0] - self.now()
                if nxt > 0:
                    self.sleep(min(nxt, 0.05))
        return self.stats()

    def stats(self):
        return summarize(self.done, self.peak_bytes, self.ticks)


def poisson_arrivals(rate, n, seed):
    """Arrival times of a Poisson process with `rate` per second."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    return np.cumsum(rng.exponential(1.0 / rate, size=n))
