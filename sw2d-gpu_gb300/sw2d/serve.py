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

The backend is injected (`batch_factory`), so the scheduling logic is
tested on the host with a fake batch.
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
        if not self.done:
            return {"requests": 0}
        served = [r for r in self.done if "error" not in r.result and not r.result.get("cancelled")]
        cancelled = sum(1 for r in self.done if r.result.get("cancelled"))
        if not served:
            return {"requests": 0, "failed": len(self.done) - cancelled, "cancelled": cancelled}
        ttr = np.array([r.finished - r.arrival for r in served])
        span = max(r.finished for r in served) - min(r.arrival for r in served)
        cu = sum(int(r.cfg.rows) * int(r.cfg.cols) * int(r.result["steps"]) for r in served)
        return {
            "requests": len(served),
            "failed": len(self.done) - len(served) - cancelled,
            "cancelled": cancelled,
            "p50_s": float(np.percentile(ttr, 50)),
            "p99_s": float(np.percentile(ttr, 99)),
            "mean_s": float(ttr.mean()),
            "scenarios_per_hour": len(self.done) / span * 3600.0 if span > 0 else None,
            "cell_updates_per_s": cu / span if span > 0 else None,
            "peak_bytes": int(self.peak_bytes),
            "ticks": self.ticks,
            "span_s": float(span),
        }


def poisson_arrivals(rate, n, seed):
    """Arrival times of a Poisson process with `rate` per second."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    return np.cumsum(rng.exponential(1.0 / rate, size=n))
