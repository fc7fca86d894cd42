"""Spatial rain distribution (sw2d_set_rain_weights): per-cell factors of the
rain rate.  The oracle's restatement on CPU, then the GPU paths against it:
FP64 bit for bit, FP32 within the FP32 bounds."""
import numpy as np
import pytest

from helpers import make_pair, max_abs, same, set_forcing


def _scenario(rows=36, cols=44, seed=5):
    from sw2d import scenarios as S
    s = S.catchment(rows, dx=10.0, seed=seed, cols=cols)
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.0, 2.0, (rows, cols))
    w[rng.random((rows, cols)) < 0.1] = 0.0  # some cells without rain
    return s, w


def _oracle(O, s, rows, cols, w=None, rain=(60.0, 120.0, 30.0)):
    o = O.Oracle(rows, cols, 10.0, 10.0, s["z"], n=s["n"], dt_mode=1, dt=1.0, south_open=1)
    o.set_state(s["h0"])
    o.set_forcing(O.OracleForcing(rain_kind=O.RAIN_LINEAR, rain=np.array(rain), rain_dt=200.0, rain_w=w))
    return o


def test_oracle_unit_weights_equal_uniform_rain(oracle_mod):
    s, _ = _scenario()
    a = _oracle(oracle_mod, s, 36, 44)
    b = _oracle(oracle_mod, s, 36, 44, w=np.ones((36, 44)))
    a.advance(10 ** 6, t_end=300.0)
    b.advance(10 ** 6, t_end=300.0)
    sa, sb = a.state(), b.state()
    for k in ("h", "um", "vn"):
        assert np.array_equal(sa[k], sb[k])
    assert a.budget()["rain_in"] == b.budget()["rain_in"]


def test_oracle_weights_scale_the_rain_budget(oracle_mod):
    """Flat, dry ground over one short step: the rain budget is the weighted
    sum of the cells' rain."""
    O = oracle_mod
    rows, cols = 20, 30
    z = np.zeros((rows, cols))
    w = np.random.default_rng(2).uniform(0.0, 3.0, (rows, cols))
    res = []
    for ww in (None, w):
        o = O.Oracle(rows, cols, 10.0, 10.0, z, dt_mode=0, dt=0.5)
        o.set_state(np.zeros((rows, cols)))
        o.set_forcing(O.OracleForcing(rain_kind=O.RAIN_STEP, rain=np.array([36.0]), rain_dt=3600.0, rain_w=ww))
        o.advance(1, 1e9)
        res.append(o.budget()["rain_in"])
    assert res[1] == pytest.approx(res[0] * w.mean(), rel=1e-12)


@pytest.mark.gpu
def test_f64_rain_weights_bitwise(oracle_mod, sw2d_mod):
    s, w = _scenario()
    o, g = make_pair(oracle_mod, sw2d_mod, 36, 44, 10.0, s["z"], s["h0"], n=s["n"], south_open=1, dt_mode=1, dt=1.0)
    o.set_forcing(oracle_mod.OracleForcing(rain_kind=oracle_mod.RAIN_LINEAR, rain=np.array([60.0, 120.0, 30.0]),
                                           rain_dt=200.0, rain_w=w))
    g.set_rain(sw2d_mod.RAIN_LINEAR, [60.0, 120.0, 30.0], 200.0)
    g.set_rain_weights(w)
    o.advance(10 ** 6, t_end=600.0)
    g.advance(10 ** 6, t_end=600.0)
    a, b = o.state(), g.state()
    for k in ("h", "um", "vn"):
        assert same(a[k], b[k]), (k, max_abs(a[k], b[k]))
    assert g.budget()["rain_in"] == pytest.approx(o.budget()["rain_in"], rel=1e-12)


@pytest.mark.gpu
def test_f64_rain_weights_times_storm(oracle_mod, sw2d_mod):
    s, w = _scenario(seed=8)
    o, g = make_pair(oracle_mod, sw2d_mod, 36, 44, 10.0, s["z"], s["h0"], n=s["n"], south_open=1, dt_mode=1, dt=1.0)
    storm = {"peak": 200.0, "x0": 0.0, "y0": 0.0, "vx": 1.0, "vy": 0.5, "sigma": 150.0}
    set_forcing(oracle_mod, o, g, storm=storm)  # the storm on both sides
    o.set_forcing(oracle_mod.OracleForcing(rain_kind=oracle_mod.RAIN_STORM, storm=storm, rain_w=w))
    g.set_rain_weights(w)
    o.advance(10 ** 6, t_end=400.0)
    g.advance(10 ** 6, t_end=400.0)
    a, b = o.state(), g.state()
    for k in ("h", "um", "vn"):
        assert same(a[k], b[k]), (k, max_abs(a[k], b[k]))


@pytest.mark.gpu
def test_f32_rain_weights_within_bounds(oracle_mod, sw2d_mod):
    s, w = _scenario(rows=64, cols=90, seed=12)
    o = _oracle(oracle_mod, s, 64, 90, w=w)
    g = sw2d_mod.Solver(rows=64, cols=90, dx=10.0, dy=10.0, precision=sw2d_mod.PREC_F32, dt_mode=1, dt=1.0,
                        south_open=1)
    g.set_static(s["z"], s["n"])
    g.set_state(s["h0"])
    g.set_rain(sw2d_mod.RAIN_LINEAR, [60.0, 120.0, 30.0], 200.0)
    g.set_rain_weights(w)
    o.advance(10 ** 6, t_end=900.0)
    g.advance(10 ** 6, t_end=900.0)
    assert max_abs(o.state()["h"], g.depth()) <= 1e-3
    assert g.budget()["rain_in"] == pytest.approx(o.budget()["rain_in"], rel=1e-4)


@pytest.mark.gpu
def test_f32_rain_weights_times_storm_within_bounds(oracle_mod, sw2d_mod):
    """The streaming kernel's form with both the rain factors and the moving
    storm (and a point source) against the oracle."""
    s, w = _scenario(rows=64, cols=90, seed=14)
    O = oracle_mod
    storm = {"peak": 200.0, "x0": 0.0, "y0": 0.0, "vx": 1.0, "vy": 0.5, "sigma": 300.0}
    cells = np.array([30 * 90 + 45], dtype=np.int32)
    q = np.array([[1.5], [0.5]])
    o = O.Oracle(64, 90, 10.0, 10.0, s["z"], n=s["n"], dt_mode=1, dt=1.0, south_open=1)
    o.set_state(s["h0"])
    o.set_forcing(O.OracleForcing(rain_kind=O.RAIN_STORM, storm=storm, rain_w=w, sources=cells, src_q=q,
                                  dtoq=300.0))
    g = sw2d_mod.Solver(rows=64, cols=90, dx=10.0, dy=10.0, precision=sw2d_mod.PREC_F32, dt_mode=1, dt=1.0,
                        south_open=1)
    g.set_static(s["z"], s["n"])
    g.set_state(s["h0"])
    g.set_storm(storm["peak"], storm["x0"], storm["y0"], storm["vx"], storm["vy"], storm["sigma"])
    g.set_point_sources(cells, q, 300.0)
    g.set_rain_weights(w)
    assert "forcing=storm/sources+rain_weights " in g.describe()
    o.advance(10 ** 6, t_end=600.0)
    g.advance(10 ** 6, t_end=600.0)
    assert max_abs(o.state()["h"], g.depth()) <= 1e-3
    assert g.budget()["rain_in"] == pytest.approx(o.budget()["rain_in"], rel=1e-4)
    assert g.budget()["source_in"] == pytest.approx(o.budget()["source_in"], rel=1e-4)


@pytest.mark.gpu
def test_rain_weights_errors_and_reset(oracle_mod, sw2d_mod):
    s, w = _scenario()
    g = sw2d_mod.Solver(rows=36, cols=44, dx=10.0, dy=10.0)
    with pytest.raises(sw2d_mod.SW2DError) as e:
        g.set_rain_weights(w)  # before sw2d_set_static
    assert e.value.status == sw2d_mod.native.ERR_STATE
    g.set_static(s["z"], s["n"])
    for bad in (-1.0, np.nan, np.inf):
        ww = w.copy()
        ww[3, 4] = bad
        with pytest.raises(sw2d_mod.SW2DError) as e:
            g.set_rain_weights(ww)
        assert e.value.status == sw2d_mod.native.ERR_INVALID_ARG
    g.close()
    # set_static clears the factors: the run is the uniform-rain run
    o, g = make_pair(oracle_mod, sw2d_mod, 36, 44, 10.0, s["z"], s["h0"], n=s["n"], south_open=1, dt_mode=1, dt=1.0)
    g.set_rain_weights(w)
    g.set_static(s["z"], s["n"])
    g.set_state(s["h0"])
    o.set_forcing(oracle_mod.OracleForcing(rain_kind=oracle_mod.RAIN_LINEAR, rain=np.array([60.0, 120.0, 30.0]),
                                           rain_dt=200.0))
    g.set_rain(sw2d_mod.RAIN_LINEAR, [60.0, 120.0, 30.0], 200.0)
    o.advance(10 ** 6, t_end=300.0)
    g.advance(10 ** 6, t_end=300.0)
    assert same(o.state()["h"], g.depth())
