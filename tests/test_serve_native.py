"""The native serving loop (sw2d_server_*): continuous batching over one
batch through the C ABI.  On the host: its defaults and the arguments it
refuses before touching the device.  On the GPU: requests submitted while
others run are admitted in order as slots and memory allow, each result is
bit-identical to the same scenario alone in a batch, and cancel/release
keep the accounting right."""
import ctypes as C

import numpy as np
import pytest


def _cfg(sw2d, rows, cols):
    return sw2d.default_config(rows=rows, cols=cols, dx=5.0, dy=5.0, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_CFL,
                               dt=2.0, cfl=0.5, south_open=1)


def _scn(seed, rows, cols):
    from sw2d import scenarios as S
    return S.catchment(rows, dx=5.0, seed=seed, cols=cols)


RAIN = np.array([0.0, 90.0, 0.0])


# ---- host only ---------------------------------------------------------------

def test_server_config_defaults():
    from sw2d import native
    c = native.server_config()
    assert c.launches_per_step == 24 and c.keep_depth == 1
    assert c.batch.max_scenarios == 1024 and c.batch.chunk == 24 and c.batch.max_bytes == 0
    c = native.server_config(max_bytes=123, launches_per_step=6, keep_depth=0)
    assert c.batch.max_bytes == 123 and c.launches_per_step == 6 and c.keep_depth == 0
    with pytest.raises(AttributeError):
        native.server_config(no_such_field=1)


def test_server_refuses_bad_arguments_without_a_device():
    from sw2d import native
    L = native.load()
    h = C.c_void_p()
    assert L.sw2d_server_create(None, C.byref(h)) == native.ERR_INVALID_ARG
    for bad in (dict(launches_per_step=0), dict(keep_depth=2)):
        c = native.server_config(**bad)
        assert L.sw2d_server_create(C.byref(c), C.byref(h)) == native.ERR_INVALID_ARG
        assert not h.value
    assert L.sw2d_server_destroy(None) == native.ERR_INVALID_ARG
    assert L.sw2d_server_step(None, None, None) == native.ERR_INVALID_ARG
    st = C.c_int32()
    assert L.sw2d_server_poll(None, 1, C.byref(st), None, None) == native.ERR_INVALID_ARG
    assert L.sw2d_server_cancel(None, 1) == native.ERR_INVALID_ARG
    assert L.sw2d_server_release(None, 1) == native.ERR_INVALID_ARG
    rid = C.c_int32()
    cfg = native.default_config(rows=4, cols=4, precision=native.PREC_F32, dt_mode=native.DT_CFL)
    assert L.sw2d_server_submit(None, C.byref(cfg), None, None, None, 0, None, 0, 1.0, 1.0,
                                C.byref(rid)) == native.ERR_INVALID_ARG
    assert L.sw2d_server_last_error(None) == b"null server"
    assert L.sw2d_server_request_error(None, 1) == b""


# ---- GPU ---------------------------------------------------------------------

def _alone(sw2d, cfg, s, t_end):
    with sw2d.Batch(chunk=6) as b:
        sid = b.add(cfg, s["z"], s["h0"], manning=s["n"], rain_kind=sw2d.RAIN_LINEAR, rain=RAIN, rain_dt=300.0,
                    t_end=t_end)
        while b.advance(12):
            pass
        return b.field(sid), b.poll()[sid]["steps"]


@pytest.mark.gpu
def test_native_server_results_equal_alone(sw2d_mod):
    shapes = [(64, 64), (90, 70), (40, 130), (128, 96), (33, 50), (70, 70)]
    ends = [240.0, 400.0, 180.0, 300.0, 500.0, 260.0]
    scns = [_scn(60 + k, r, c) for k, (r, c) in enumerate(shapes)]
    with sw2d_mod.ServerHandle(chunk=6, launches_per_step=6) as srv:
        ids = []

        def submit(k):
            r, c = shapes[k]
            ids.append(srv.submit(_cfg(sw2d_mod, r, c), scns[k]["z"], scns[k]["h0"], manning=scns[k]["n"],
                                  rain_kind=sw2d_mod.RAIN_LINEAR, rain=RAIN, rain_dt=300.0, t_end=ends[k]))

        for k in range(3):
            submit(k)
        assert srv.poll(ids[0])["state"] == sw2d_mod.REQ_PENDING
        srv.step()
        srv.step()
        assert srv.poll(ids[0])["state"] == sw2d_mod.REQ_RUNNING and srv.poll(ids[0])["steps"] == 12
        for k in range(3, len(shapes)):  # arrive while the first ones run
            submit(k)
        steps = 0
        while True:
            pending, running = srv.step()
            steps += 1
            if pending == 0 and running == 0:
                break
            assert steps < 2000
        assert srv.bytes_in_use() == 0
        for k, rid in enumerate(ids):
            st = srv.poll(rid)
            assert st["state"] == sw2d_mod.REQ_DONE
            assert abs(st["t"] - ends[k]) < 1e-6
            depth, n = _alone(sw2d_mod, _cfg(sw2d_mod, *shapes[k]), scns[k], ends[k])
            assert st["steps"] == n
            assert np.array_equal(srv.depth(rid), depth), shapes[k]
            bud = srv.budget(rid)
            assert bud["steps"] == n and bud["rain_in"] > 0
            srv.release(rid)
            assert srv.poll(rid)["state"] == sw2d_mod.REQ_UNKNOWN


@pytest.mark.gpu
def test_native_server_admits_by_memory_and_slots(sw2d_mod):
    s = _scn(70, 64, 64)
    cfg = _cfg(sw2d_mod, 64, 64)
    need = sw2d_mod.batch_scenario_bytes(cfg, 3, True)
    with sw2d_mod.ServerHandle(chunk=6, launches_per_step=6, max_bytes=int(need * 2.5)) as srv:
        big = _cfg(sw2d_mod, 200, 200)
        sb = _scn(71, 200, 200)
        with pytest.raises(sw2d_mod.SW2DError) as e:  # more than the whole budget
            srv.submit(big, sb["z"], sb["h0"], manning=sb["n"], rain_kind=sw2d_mod.RAIN_LINEAR, rain=RAIN,
                       rain_dt=300.0, t_end=100.0)
        assert e.value.status == 1
        ids = [srv.submit(cfg, s["z"], s["h0"], manning=s["n"], rain_kind=sw2d_mod.RAIN_LINEAR, rain=RAIN,
                          rain_dt=300.0, t_end=60.0 + 30.0 * k) for k in range(5)]
        pending, running = srv.step()
        assert (pending, running) == (3, 2)
        assert [srv.poll(i)["state"] for i in ids] == [sw2d_mod.REQ_RUNNING] * 2 + [sw2d_mod.REQ_PENDING] * 3
        seen_max = 0
        for _ in range(2000):
            pending, running = srv.step()
            seen_max = max(seen_max, running)
            assert srv.bytes_in_use() <= int(need * 2.5)
            if pending == 0 and running == 0:
                break
        assert seen_max <= 2
        assert all(srv.poll(i)["state"] == sw2d_mod.REQ_DONE for i in ids)
    # one scenario slot: requests run one at a time, in submission order
    with sw2d_mod.ServerHandle(chunk=6, launches_per_step=6, max_scenarios=1) as srv:
        ids = [srv.submit(cfg, s["z"], s["h0"], manning=s["n"], rain_kind=sw2d_mod.RAIN_LINEAR, rain=RAIN,
                          rain_dt=300.0, t_end=40.0) for _ in range(3)]
        order = []
        for _ in range(1000):
            pending, running = srv.step()
            for i in ids:
                if srv.poll(i)["state"] == sw2d_mod.REQ_DONE and i not in order:
                    order.append(i)
            if pending == 0 and running == 0:
                break
        assert order == ids


@pytest.mark.gpu
def test_native_server_cancel_release_and_keep_depth(sw2d_mod):
    s = _scn(80, 48, 48)
    cfg = _cfg(sw2d_mod, 48, 48)
    with sw2d_mod.ServerHandle(chunk=6, launches_per_step=6, max_scenarios=1, keep_depth=0) as srv:
        a, b, c = [srv.submit(cfg, s["z"], s["h0"], manning=s["n"], rain_kind=sw2d_mod.RAIN_LINEAR, rain=RAIN,
                              rain_dt=300.0, t_end=1e6) for _ in range(3)]
        assert srv.step() == (2, 1)
        with pytest.raises(sw2d_mod.SW2DError):  # not finished
            srv.release(a)
        srv.cancel(b)  # pending
        assert srv.poll(b)["state"] == sw2d_mod.REQ_CANCELLED
        used = srv.bytes_in_use()
        assert used > 0
        srv.cancel(a)  # running: leaves the batch, memory back
        assert srv.poll(a)["state"] == sw2d_mod.REQ_CANCELLED and srv.bytes_in_use() == 0
        with pytest.raises(sw2d_mod.SW2DError):
            srv.cancel(a)
        assert srv.step() == (0, 1)  # c takes the freed slot
        assert srv.poll(c)["state"] == sw2d_mod.REQ_RUNNING and srv.bytes_in_use() == used
        srv.cancel(c)
        for rid in (a, b, c):
            srv.release(rid)
            assert srv.poll(rid)["state"] == sw2d_mod.REQ_UNKNOWN
        d = srv.submit(cfg, s["z"], s["h0"], manning=s["n"], rain_kind=sw2d_mod.RAIN_LINEAR, rain=RAIN,
                       rain_dt=300.0, t_end=30.0)
        for _ in range(1000):
            if srv.step() == (0, 0):
                break
        assert srv.poll(d)["state"] == sw2d_mod.REQ_DONE
        assert srv.budget(d)["steps"] > 0
        with pytest.raises(sw2d_mod.SW2DError):  # keep_depth = 0: no raster kept
            srv.depth(d)


@pytest.mark.gpu
def test_native_server_request_refused_at_admission_fails_alone(sw2d_mod):
    """A request whose work units do not fit the batch's unit table is refused
    by the batch at admission: it fails alone, with the batch's reason, its
    device memory goes back, and the request behind it is served."""
    from sw2d import native
    small, big = _scn(90, 64, 64), _scn(91, 128, 128)
    with sw2d_mod.ServerHandle(chunk=6, launches_per_step=6, max_units=30) as srv:  # 12 units fit, 40 do not
        rb = srv.submit(_cfg(sw2d_mod, 128, 128), big["z"], big["h0"], manning=big["n"],
                        rain_kind=sw2d_mod.RAIN_LINEAR, rain=RAIN, rain_dt=300.0, t_end=60.0)
        rs = srv.submit(_cfg(sw2d_mod, 64, 64), small["z"], small["h0"], manning=small["n"],
                        rain_kind=sw2d_mod.RAIN_LINEAR, rain=RAIN, rain_dt=300.0, t_end=60.0)
        for _ in range(1000):
            if srv.step() == (0, 0):
                break
        assert srv.poll(rb)["state"] == sw2d_mod.REQ_FAILED
        assert "unit table" in srv.request_error(rb)
        assert srv.poll(rs)["state"] == sw2d_mod.REQ_DONE
        b = C.c_void_p()
        assert native.load().sw2d_server_get_batch(srv._h, C.byref(b)) == native.OK
        used = C.c_int64()
        assert native.load().sw2d_batch_bytes_in_use(b, C.byref(used)) == native.OK
        assert used.value == 0 and srv.bytes_in_use() == 0
