"""Batched scenarios (sw2d_batch_*): uneven sizes in one persistent launch
per iteration, each with its own CFL step, forcing and end time.

Each scenario must advance exactly as it would alone: bit-identical depth
and discharges against the single-scenario FP32 handle, and against the
same scenario alone in a batch, whatever else is in the mix and whenever it
was admitted."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scn(seed, rows, cols, dx=5.0):
    from sw2d import scenarios as S
    s = S.catchment(rows, dx=dx, seed=seed, cols=cols)
    return s


def _cfg(sw2d, rows, cols, dx=5.0, **kw):
    return sw2d.default_config(rows=rows, cols=cols, dx=dx, dy=dx, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_CFL,
                               dt=2.0, cfl=0.5, south_open=1, **kw)


def _rain(peak):
    return np.array([0.0, peak, 0.0]), 300.0  # triangular hyetograph, 600 s


def test_batched_equals_single_handle(sw2d_mod):
    s = _scn(1, 90, 70)
    knots, kdt = _rain(120.0)
    single = sw2d_mod.Solver(_cfg(sw2d_mod, 90, 70))
    single.set_static(s["z"], s["n"])
    single.set_state(s["h0"])
    single.set_rain(sw2d_mod.RAIN_LINEAR, knots, kdt)
    single.advance(100, t_end=900.0)
    with sw2d_mod.Batch(chunk=6) as b:
        sid = b.add(_cfg(sw2d_mod, 90, 70), s["z"], s["h0"], manning=s["n"], rain_kind=sw2d_mod.RAIN_LINEAR,
                    rain=knots, rain_dt=kdt, t_end=900.0)
        b.advance(100)
        st = b.poll()[sid]
        assert st["steps"] == 100
        assert np.array_equal(b.field(sid), single.depth())
        assert np.array_equal(b.field(sid, sw2d_mod.FIELD_UM), single.field(sw2d_mod.FIELD_UM))
        assert np.array_equal(b.field(sid, sw2d_mod.FIELD_VN), single.field(sw2d_mod.FIELD_VN))
        assert st["t"] == single.budget()["t"]


def test_alone_equals_in_the_mix(sw2d_mod):
    shapes = [(64, 64), (130, 75), (33, 200), (96, 96)]
    scns = [_scn(10 + k, r, c) for k, (r, c) in enumerate(shapes)]
    alone = []
    for k, (r, c) in enumerate(shapes):
        knots, kdt = _rain(40.0 + 30.0 * k)
        with sw2d_mod.Batch(chunk=6) as b:
            sid = b.add(_cfg(sw2d_mod, r, c), scns[k]["z"], scns[k]["h0"], manning=scns[k]["n"],
                        rain_kind=sw2d_mod.RAIN_LINEAR, rain=knots, rain_dt=kdt, t_end=1200.0)
            b.advance(90)
            alone.append(b.field(sid))
    with sw2d_mod.Batch(chunk=6) as b:
        ids = []
        for k, (r, c) in enumerate(shapes):
            knots, kdt = _rain(40.0 + 30.0 * k)
            ids.append(b.add(_cfg(sw2d_mod, r, c), scns[k]["z"], scns[k]["h0"], manning=scns[k]["n"],
                             rain_kind=sw2d_mod.RAIN_LINEAR, rain=knots, rain_dt=kdt, t_end=1200.0))
        b.advance(90)
        for k, sid in enumerate(ids):
            assert np.array_equal(b.field(sid), alone[k]), shapes[k]


def test_admit_and_retire_mid_run(sw2d_mod):
    a, c = _scn(21, 80, 60), _scn(22, 50, 90)
    knots, kdt = _rain(100.0)
    with sw2d_mod.Batch(chunk=6) as ref:
        rc = ref.add(_cfg(sw2d_mod, 50, 90), c["z"], c["h0"], manning=c["n"], rain_kind=sw2d_mod.RAIN_LINEAR,
                     rain=knots, rain_dt=kdt, t_end=1e9)
        ref.advance(61)
        expect_c = ref.field(rc)
    with sw2d_mod.Batch(chunk=6) as b:
        ia = b.add(_cfg(sw2d_mod, 80, 60), a["z"], a["h0"], manning=a["n"], rain_kind=sw2d_mod.RAIN_LINEAR,
                   rain=knots, rain_dt=kdt, t_end=1e9)
        b.advance(31)  # odd count: the next admission lands on another clock parity
        ic = b.add(_cfg(sw2d_mod, 50, 90), c["z"], c["h0"], manning=c["n"], rain_kind=sw2d_mod.RAIN_LINEAR,
                   rain=knots, rain_dt=kdt, t_end=1e9)
        b.advance(20)
        used = b.bytes_in_use()
        b.remove(ia)
        assert b.bytes_in_use() < used
        b.advance(41)
        st = b.poll()
        assert ia not in st and st[ic]["steps"] == 61
        assert np.array_equal(b.field(ic), expect_c)


def test_uneven_end_times_and_budgets(sw2d_mod):
    shapes = [(40, 40), (120, 64), (64, 150)]
    ends = [300.0, 600.0, 450.0]
    with sw2d_mod.Batch(chunk=12) as b:
        ids = []
        for k, (r, c) in enumerate(shapes):
            s = _scn(30 + k, r, c)
            knots, kdt = _rain(80.0)
            ids.append(b.add(_cfg(sw2d_mod, r, c), s["z"], s["h0"], manning=s["n"], rain_kind=sw2d_mod.RAIN_LINEAR,
                             rain=knots, rain_dt=kdt, t_end=ends[k]))
        running = len(ids)
        loops = 0
        while running and loops < 500:
            running = b.advance(24)
            loops += 1
        st = b.poll()
        for k, sid in enumerate(ids):
            assert not st[sid]["running"]
            assert abs(st[sid]["t"] - ends[k]) < 1e-6
            bud = b.budget(sid)
            rhs = bud["rain_in"] - bud["outflow"] + bud["clamp_gain"]
            assert abs(bud["volume"] - rhs) <= 1e-5 * max(bud["rain_in"], 1e-12)


def test_memory_budget_refuses_admission(sw2d_mod):
    s = _scn(40, 64, 64)
    need = sw2d_mod.batch_scenario_bytes(_cfg(sw2d_mod, 64, 64), 3, True)
    with sw2d_mod.Batch(chunk=6, max_bytes=int(need * 1.5)) as b:
        knots, kdt = _rain(50.0)
        b.add(_cfg(sw2d_mod, 64, 64), s["z"], s["h0"], manning=s["n"], rain_kind=sw2d_mod.RAIN_LINEAR, rain=knots,
              rain_dt=kdt, t_end=100.0)
        with pytest.raises(sw2d_mod.SW2DError) as e:
            b.add(_cfg(sw2d_mod, 64, 64), s["z"], s["h0"], manning=s["n"], rain_kind=sw2d_mod.RAIN_LINEAR,
                  rain=knots, rain_dt=kdt, t_end=100.0)
        assert e.value.status == 2  # SW2D_ERR_OOM
