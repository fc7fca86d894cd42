"""The serving loop's scheduling on the host, with a fake batch: admission
by footprint in arrival order, waiting for memory, retirement, statistics."""
import numpy as np
import pytest


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += dt


class FakeBatch:
    """Each scenario runs for `steps_needed` launches; time advances by
    `tick_cost` per advance."""

    def __init__(self, clock, tick_cost=0.1):
        self.clock, self.tick_cost = clock, tick_cost
        self.scen, self.next_id, self.adds, self.removes = {}, 0, [], []

    def add(self, cfg, z, depth, manning=None, rain_kind=0, rain=None, rain_dt=1.0, t_end=1e300):
        sid = self.next_id
        self.next_id += 1
        self.scen[sid] = {"left": int(t_end), "steps": 0}
        self.adds.append((sid, self.clock.t))
        return sid

    def advance(self, launches, wait=True):
        self.clock.t += self.tick_cost
        for s in self.scen.values():
            k = min(launches, s["left"])
            s["left"] -= k
            s["steps"] += k

    def poll(self):
        return {sid: {"running": s["left"] > 0, "t": float(s["steps"]), "steps": s["steps"]}
                for sid, s in self.scen.items()}

    def budget(self, sid):
        return {"volume": 0.0}

    def field(self, sid, which=0):
        return np.zeros((1, 1))

    def remove(self, sid):
        self.removes.append((sid, self.clock.t))
        del self.scen[sid]


class Cfg:
    rows = 10
    cols = 10


def _req(serve, rid, arrival, steps, nbytes):
    r = serve.Request(rid=rid, arrival=arrival, cfg=Cfg(), z=None, depth=None, manning=None, rain_kind=0, rain=None,
                      rain_dt=1.0, t_end=float(steps))
    r._bytes = nbytes
    return r


def test_admission_respects_memory_and_order():
    from sw2d import serve
    clk = FakeClock()
    fb = FakeBatch(clk)
    srv = serve.Server(lambda: fb, bytes_of=lambda r: r._bytes, max_bytes=100, launches_per_tick=10, clock=clk,
                       sleep=clk.sleep)
    reqs = [_req(serve, 0, 0.0, 30, 60), _req(serve, 1, 0.0, 10, 60), _req(serve, 2, 0.0, 10, 30)]
    st = srv.run(reqs)
    assert st["requests"] == 3
    assert srv.peak_bytes <= 100
    # request 1 (60 B) cannot join request 0 (60 B); request 2 (30 B) can
    first_tick = [sid for sid, t in fb.adds if t == 0.0]
    assert first_tick == [0, 1] or first_tick == [0, 2]
    admitted = {r.rid: r.admitted for r in srv.done}
    assert admitted[0] == 0.0 and admitted[2] == 0.0 and admitted[1] > 0.0
    for r in srv.done:
        assert r.finished >= r.admitted >= r.arrival


def test_requests_wait_for_arrival_and_stats():
    from sw2d import serve
    clk = FakeClock()
    fb = FakeBatch(clk, tick_cost=0.05)
    srv = serve.Server(lambda: fb, bytes_of=lambda r: 10, max_bytes=1000, launches_per_tick=5, clock=clk,
                       sleep=clk.sleep)
    arr = serve.poisson_arrivals(rate=4.0, n=20, seed=3)
    reqs = [_req(serve, k, float(a), 20, 10) for k, a in enumerate(arr)]
    st = srv.run(reqs)
    assert st["requests"] == 20
    for r in srv.done:
        assert r.admitted >= r.arrival
        assert r.result["steps"] == 20
    assert 0 < st["p50_s"] <= st["p99_s"]
    assert len(fb.scen) == 0 and srv.bytes_used == 0


def test_oversized_request_rejected():
    from sw2d import serve
    clk = FakeClock()
    srv = serve.Server(lambda: FakeBatch(clk), bytes_of=lambda r: 500, max_bytes=100, clock=clk, sleep=clk.sleep)
    with pytest.raises(ValueError):
        srv.submit(_req(serve, 0, 0.0, 5, 500))


def test_poisson_arrivals_rate():
    from sw2d import serve
    a = serve.poisson_arrivals(rate=10.0, n=5000, seed=1)
    assert np.all(np.diff(a) > 0)
    assert abs(len(a) / a[-1] - 10.0) < 0.5


def test_admission_waits_for_a_free_scenario_slot():
    """A batch with fewer scenario slots than the memory budget admits: the
    extra requests wait for a slot instead of failing in batch.add."""
    from sw2d import serve
    clk = FakeClock()
    fb = FakeBatch(clk)

    class Slots:
        max_scenarios = 2

    fb.cfg = Slots()
    real_add = fb.add

    def add(*a, **k):
        assert len(fb.scen) < 2, "the server overfilled the scenario table"
        return real_add(*a, **k)

    fb.add = add
    srv = serve.Server(lambda: fb, bytes_of=lambda r: r._bytes, max_bytes=1000, launches_per_tick=10, clock=clk,
                       sleep=clk.sleep)
    st = srv.run([_req(serve, k, 0.0, 20, 10) for k in range(5)])
    assert st["requests"] == 5 and st["failed"] == 0


def test_a_refused_request_fails_alone():
    """A request the library refuses (here: batch.add raises) finishes with
    an error; the others are served."""
    from sw2d import serve
    from sw2d.native import SW2DError
    clk = FakeClock()
    fb = FakeBatch(clk)
    real_add = fb.add

    def add(cfg, z, depth, **k):
        if k["t_end"] == 7.0:
            raise SW2DError(1, "sw2d_batch_add")
        return real_add(cfg, z, depth, **k)

    fb.add = add
    srv = serve.Server(lambda: fb, bytes_of=lambda r: r._bytes, max_bytes=100, launches_per_tick=10, clock=clk,
                       sleep=clk.sleep)
    reqs = [_req(serve, 0, 0.0, 20, 10), _req(serve, 1, 0.0, 7, 10), _req(serve, 2, 0.5, 20, 10)]
    st = srv.run(reqs)
    assert st["requests"] == 2 and st["failed"] == 1
    bad = [r for r in srv.done if "error" in r.result]
    assert [r.rid for r in bad] == [1] and "sw2d_batch_add" in bad[0].result["error"]
    assert srv.bytes_used == 0 and not srv.running


def test_poll_and_cancel():
    """submit / poll / cancel: a pending request leaves the queue, a running
    one leaves the batch and returns its memory; the rest are served."""
    from sw2d import serve
    clk = FakeClock()
    fb = FakeBatch(clk)
    srv = serve.Server(lambda: fb, bytes_of=lambda r: r._bytes, max_bytes=100, launches_per_tick=10, clock=clk,
                       sleep=clk.sleep)
    for r in (_req(serve, 0, 0.0, 50, 40), _req(serve, 1, 0.0, 50, 40), _req(serve, 2, 5.0, 50, 40)):
        srv.submit(r)
    assert [srv.poll(k) for k in (0, 1, 2, 9)] == ["pending", "pending", "pending", None]
    srv.step()  # starts the clock, admits 0 and 1 (80 of 100 bytes); 2 arrives later
    assert srv.poll(0) == "running" and srv.poll(2) == "pending" and srv.bytes_used == 80
    assert srv.cancel(1) and srv.poll(1) == "cancelled" and srv.bytes_used == 40
    assert [sid for sid, _ in fb.removes] == [1]
    assert srv.cancel(2) and srv.poll(2) == "cancelled" and not srv.pending
    assert not srv.cancel(1) and not srv.cancel(9)
    while srv.pending or srv.running:
        srv.step()
    st = srv.stats()
    assert srv.poll(0) == "done"
    assert st["requests"] == 1 and st["cancelled"] == 2 and st["failed"] == 0


class FakeServerHandle:
    """Stands in for ServerHandle with the native loop's rules: submission
    order, admission while `slots` and `budget` allow, `launches` per step,
    a request's end after `t_end` launches; time advances by tick_cost."""

    def __init__(self, clock, slots=2, budget=100, launches=10, tick_cost=0.1):
        self.clock, self.slots, self.limit, self.launches, self.tick_cost = clock, slots, budget, launches, tick_cost
        self.req, self.queue, self.next_id, self.used, self.released = {}, [], 1, 0, []

    def submit(self, cfg, z, depth, manning=None, rain_kind=0, rain=None, rain_dt=1.0, t_end=1e300):
        from sw2d import SW2DError
        nbytes = getattr(cfg, "nbytes", 10)
        if nbytes > self.limit:
            raise SW2DError(1, "the request needs more device memory than the whole budget")
        rid = self.next_id
        self.next_id += 1
        self.req[rid] = {"state": 1, "left": int(t_end), "steps": 0, "bytes": nbytes}
        self.queue.append(rid)
        return rid

    def step(self):
        running = [r for r, v in self.req.items() if v["state"] == 2]
        for rid in list(self.queue):
            v = self.req[rid]
            if len(running) < self.slots and self.used + v["bytes"] <= self.limit:
                v["state"] = 2
                self.used += v["bytes"]
                running.append(rid)
                self.queue.remove(rid)
        self.clock.t += self.tick_cost
        for rid in running:
            v = self.req[rid]
            k = min(self.launches, v["left"])
            v["left"] -= k
            v["steps"] += k
            if v["left"] == 0:
                v["state"] = 3
                self.used -= v["bytes"]
        return len(self.queue), sum(1 for v in self.req.values() if v["state"] == 2)

    def poll(self, rid):
        v = self.req.get(rid)
        return {"state": v["state"] if v else 0, "t": float(v["steps"]) if v else 0.0, "steps": v["steps"] if v else 0}

    def budget(self, rid):
        return {"steps": self.req[rid]["steps"]}

    def depth(self, rid):
        return np.full((1, 1), float(rid))

    def request_error(self, rid):
        return ""

    def release(self, rid):
        self.released.append(rid)
        del self.req[rid]

    def bytes_in_use(self):
        return self.used


def test_native_driver_submits_on_arrival_and_collects():
    from sw2d import serve
    clk = FakeClock()
    fh = FakeServerHandle(clk, slots=2, budget=100, launches=10)
    srv = serve.NativeServer(lambda: fh, keep_results=lambda r: r.rid % 2 == 0, clock=clk, sleep=clk.sleep)
    arr = [0.0, 0.0, 0.0, 0.35, 2.0]
    reqs = [_req(serve, k, a, 20 + 10 * k, 10) for k, a in enumerate(arr)]
    big = _req(serve, 9, 0.5, 10, 10)
    big.cfg = type("BigCfg", (), {"rows": 10, "cols": 10, "nbytes": 500})()
    st = srv.run(reqs + [big])
    assert st["requests"] == 5 and st["failed"] == 1
    assert not srv.active and not srv.pending and sorted(fh.released) == [1, 2, 3, 4, 5]
    for r in srv.done:
        if r.rid == 9:
            assert "error" in r.result
            continue
        assert r.finished >= r.admitted >= r.arrival
        assert r.result["steps"] == r.t_end
        assert ("depth" in r.result) == (r.rid % 2 == 0)
    # two slots: the third request waits for the first to finish
    third = next(r for r in srv.done if r.rid == 2)
    first = next(r for r in srv.done if r.rid == 0)
    assert third.admitted >= first.finished
    assert srv.peak_bytes <= 100 and st["p50_s"] <= st["p99_s"]
