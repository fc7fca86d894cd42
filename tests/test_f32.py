"""FP32 paths (warp-streaming kernel, shared-memory tile kernel) against the
FP64 oracle and against each other, through the C ABI.

Stated bounds for the FP32 state: max |dh| <= 1 mm against the FP64 oracle
and flooded area (h > th) within 0.1 %, on rain-runoff scenarios; the
relative volume-conservation error of the FP64 budget <= 1e-6.
"""
import numpy as np
import pytest

from helpers import make_pair, max_abs, set_forcing

pytestmark = pytest.mark.gpu

TH = 1.0e-4
TOL_MM = 1.0e-3


def _f32(sw2d, rows, cols, dx, z, h0, n=None, kernel=0, strip_h=0, **kw):
    g = sw2d.Solver(rows=rows, cols=cols, dx=dx, dy=dx, precision=sw2d.PREC_F32, kernel=kernel, strip_h=strip_h,
                    **kw)
    g.set_static(z, n)
    g.set_state(h0)
    return g


def _catchment(seed=3, rows=96, cols=80, holes=True):
    from sw2d import scenarios as S
    s = S.catchment(rows, dx=5.0, seed=seed, cols=cols)
    z = s["z"].copy()
    if holes:
        rng = np.random.default_rng(seed)
        z[rng.random(z.shape) < 0.02] = -9999.0
    return s, z


def _flooded_area_rel(a, b):
    na, nb = np.count_nonzero(a > TH), np.count_nonzero(b > TH)
    return abs(na - nb) / max(na, 1)


@pytest.mark.parametrize("kernel", [1, 2])
def test_f32_catchment_rain_vs_oracle(oracle_mod, sw2d_mod, kernel):
    s, z = _catchment()
    o, g64 = make_pair(oracle_mod, sw2d_mod, 96, 80, 5.0, z, s["h0"], n=s["n"], south_open=1, dt_mode=1, dt=2.0)
    g64.close()
    g = _f32(sw2d_mod, 96, 80, 5.0, z, s["h0"], n=s["n"], kernel=kernel, south_open=1, dt_mode=1, dt=2.0)
    set_forcing(oracle_mod, o, g, rain_kind=2, rain=np.array([100.0, 50.0]), rain_dt=600.0)
    o.advance(10 ** 6, t_end=1200.0)
    g.advance(10 ** 6, t_end=1200.0)
    a, b = o.state()["h"], g.depth()
    err = max_abs(a, b)
    print("max |dh| =", err, "flooded-area rel diff =", _flooded_area_rel(a, b))
    assert err <= TOL_MM
    assert _flooded_area_rel(a, b) <= 1e-3
    bud = g.budget()
    rhs = bud["volume0"] + bud["rain_in"] + bud["source_in"] - bud["evap_out"] - bud["outflow"] + bud["clamp_gain"]
    vol_err = abs(bud["volume"] - rhs) / bud["volume"]
    print("relative volume error", vol_err)
    assert vol_err <= 1e-6


def test_stream_matches_tile_kernel(sw2d_mod):
    """Same scheme, same precision, two kernel organisations.  The streaming
    kernel forms the bed slopes from face differences taken in FP64, the tile
    kernel from FP32 elevations, so they agree to the FP32 bound, not to the
    last bit."""
    s, z = _catchment(seed=4, rows=70, cols=130)
    g1 = _f32(sw2d_mod, 70, 130, 5.0, z, s["h0"], n=s["n"], kernel=1, south_open=1, dt_mode=1, dt=2.0)
    g2 = _f32(sw2d_mod, 70, 130, 5.0, z, s["h0"], n=s["n"], kernel=2, south_open=1, dt_mode=1, dt=2.0, strip_h=16)
    for g in (g1, g2):
        g.set_rain(sw2d_mod.RAIN_STEP, [150.0], 3600.0)
        assert g.advance(300) == 300
    b1, b2 = g1.budget(), g2.budget()
    assert abs(b1["t"] - b2["t"]) <= 1e-6 * b1["t"]
    assert max_abs(g1.depth(), g2.depth()) <= TOL_MM


@pytest.mark.parametrize("strip_h", [1, 7, 16, 64, 128])
def test_stream_strip_heights_agree(sw2d_mod, strip_h):
    """The strip decomposition must not change the result (up to FP32
    contraction differences, there are none: same code per cell)."""
    s, z = _catchment(seed=6, rows=50, cols=60)
    ref = _f32(sw2d_mod, 50, 60, 5.0, z, s["h0"], n=s["n"], kernel=2, strip_h=50, dt_mode=1, dt=2.0)
    g = _f32(sw2d_mod, 50, 60, 5.0, z, s["h0"], n=s["n"], kernel=2, strip_h=strip_h, dt_mode=1, dt=2.0)
    for x in (ref, g):
        x.set_rain(sw2d_mod.RAIN_STEP, [200.0], 3600.0)
        x.advance(120)
    assert np.array_equal(ref.depth(), g.depth())


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 5])
def test_stream_variants_agree(sw2d_mod, variant):
    """Every build of the streaming kernel (CTA size, register budget, row-loop
    unrolling) gives the same bits as variant 0, on a grid with interior and
    edge units, per-cell n, a moving storm, point sources and an open south
    edge."""
    from sw2d import scenarios as S
    rows, cols = 150, 170
    s = S.catchment(rows, dx=10.0, seed=21, cols=cols)
    cells = np.array([20 * cols + 40, 75 * cols + 90, 140 * cols + 3], dtype=np.int32)
    q = np.array([[1.0, 2.0, 0.5], [3.0, 0.0, 1.0]])
    out = []
    for v in (0, variant):
        g = _f32(sw2d_mod, rows, cols, 10.0, s["z"], s["h0"], n=s["n"], kernel=2, strip_h=16, variant=v,
                 south_open=1, dt_mode=1, dt=2.0)
        g.set_storm(150.0, 0.0, 0.0, 2.0, 1.0, 600.0)
        g.set_point_sources(cells, q, 300.0)
        g.advance(150)
        out.append((g.depth(), g.state(), g.budget()))
        g.close()
    (d0, s0, b0), (d1, s1, b1) = out
    assert np.array_equal(d0, d1)
    assert np.array_equal(s0["um"], s1["um"]) and np.array_equal(s0["vn"], s1["vn"])
    assert b0["t"] == b1["t"]


def test_stream_skewed_strips_agree(sw2d_mod):
    """Strip heights skewed toward the strips launched first (the library's
    choice for one launch per iteration over a full wave of resident warps)
    give the same bits as strips of equal height."""
    from sw2d import scenarios as S
    n = 2048
    s = S.catchment(n, dx=5.0, seed=2)
    out = []
    for strip_h in (0, 26):  # one full wave (skewed); two waves (even)
        g = _f32(sw2d_mod, n, n, 5.0, s["z"], s["h0"], n=s["n"], kernel=2, strip_h=strip_h, south_open=1, dt_mode=1,
                 dt=2.0)
        g.set_rain(sw2d_mod.RAIN_STEP, [80.0], 3600.0)
        assert ("strip_skew=" in g.describe()) == (strip_h == 0), g.describe()
        assert g.advance(24) == 24
        out.append((g.depth(), g.state()))
        g.close()
    (d0, s0), (d1, s1) = out
    assert np.array_equal(d0, d1)
    assert np.array_equal(s0["um"], s1["um"]) and np.array_equal(s0["vn"], s1["vn"])


@pytest.mark.parametrize("raster", [True, False])
def test_stream_tma_build_agrees(sw2d_mod, raster):
    """The build that stages rows in shared memory by TMA (variant 6, uniform
    forcing only) gives the same bits as variant 0: per-cell or scalar n,
    NODATA holes, step rain with runoff fractions and evaporation, an open
    south edge, CFL steps, over strips whose first rows read remainder rows
    above the frame (TMA's zero fill) and a last, shorter strip."""
    rows, cols = 150, 170
    s, z = _catchment(seed=8, rows=rows, cols=cols)
    out = []
    for v in (0, 6):
        g = _f32(sw2d_mod, rows, cols, 5.0, z, s["h0"], n=s["n"] if raster else None, kernel=2, strip_h=16,
                 variant=v, south_open=1, dt_mode=1, dt=2.0, manning=0.04, INT=0.2, INF=0.1, LWL=0.01,
                 EV_WL_min=0.002)
        g.set_rain(sw2d_mod.RAIN_STEP, [120.0, 30.0], 300.0)
        g.set_evaporation([2.0e-7], 3600.0)
        assert ("tma" in g.describe()) == (v == 6)
        g.advance(150)
        out.append((g.depth(), g.state(), g.budget()))
        g.close()
    (d0, s0, b0), (d1, s1, b1) = out
    assert np.array_equal(d0, d1)
    assert np.array_equal(s0["um"], s1["um"]) and np.array_equal(s0["vn"], s1["vn"])
    assert b0["t"] == b1["t"] and b0["volume"] == b1["volume"]


@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (9, 1), (17, 33), (33, 17), (3, 65), (40, 26), (5, 50), (7, 57),
                                   (6, 113)])
def test_stream_ragged_grids_vs_oracle(oracle_mod, sw2d_mod, shape):
    rows, cols = shape
    rng = np.random.default_rng(rows * 100 + cols)
    z = rng.uniform(0, 0.5, (rows, cols))
    h0 = rng.uniform(0, 1.0, (rows, cols)) * (rng.random((rows, cols)) < 0.6)
    o = oracle_mod.Oracle(rows, cols, 1.0, 1.0, z, dt_mode=0, dt=0.02)
    o.set_state(h0)
    g = _f32(sw2d_mod, rows, cols, 1.0, z, h0, kernel=2, dt_mode=0, dt=0.02)
    o.advance(40, 1e9)
    g.advance(40, 1e9)
    assert max_abs(o.state()["h"], g.depth()) <= TOL_MM


def test_stream_sources_storm_open_south(oracle_mod, sw2d_mod):
    from sw2d import scenarios as S
    rows, cols = 64, 72
    s = S.catchment(rows, dx=20.0, seed=13, cols=cols, manning=0.05)
    o, g64 = make_pair(oracle_mod, sw2d_mod, rows, cols, 20.0, s["z"], s["h0"], manning=0.05, south_open=1,
                       dt_mode=1, dt=5.0)
    g64.close()
    g = _f32(sw2d_mod, rows, cols, 20.0, s["z"], s["h0"], manning=0.05, kernel=2, south_open=1, dt_mode=1, dt=5.0)
    storm = {"peak": 200.0, "x0": 0.0, "y0": 0.0, "vx": 1.5, "vy": 1.0, "sigma": 400.0}
    cells = np.array([10 * cols + 30, 40 * cols + 5, 40 * cols + 5], dtype=np.int32)
    q = np.array([[2.0, 1.0, 3.0], [4.0, 0.5, 1.0], [1.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    set_forcing(oracle_mod, o, g, storm=storm, sources=cells, src_q=q, dtoq=200.0)
    o.advance(10 ** 6, t_end=600.0)
    g.advance(10 ** 6, t_end=600.0)
    a, b = o.state()["h"], g.depth()
    print("max |dh| =", max_abs(a, b))
    assert max_abs(a, b) <= TOL_MM
    bo, bg = o.budget(), g.budget()
    assert bg["source_in"] == pytest.approx(bo["source_in"], rel=1e-4)
    assert bg["rain_in"] == pytest.approx(bo["rain_in"], rel=1e-4)
    assert bg["outflow"] == pytest.approx(bo["outflow"], rel=1e-3, abs=1e-3)


def test_stream_forcing_forms_switch_mid_run(oracle_mod, sw2d_mod):
    """The streaming kernel has a form for uniform rain and one carrying the
    moving storm and the point sources; the launcher picks the form from the
    handle's forcing whenever the launch graph is captured.  A run that goes
    uniform rain -> storm with point sources -> uniform rain again (sources
    cleared) follows the oracle through both forms and back."""
    from sw2d import scenarios as S
    O = oracle_mod
    rows, cols = 64, 72
    s = S.catchment(rows, dx=20.0, seed=17, cols=cols, manning=0.05)
    o, g64 = make_pair(O, sw2d_mod, rows, cols, 20.0, s["z"], s["h0"], manning=0.05, south_open=1, dt_mode=1,
                       dt=5.0)
    g64.close()
    g = _f32(sw2d_mod, rows, cols, 20.0, s["z"], s["h0"], manning=0.05, kernel=2, south_open=1, dt_mode=1, dt=5.0)
    rain = np.array([40.0])
    set_forcing(O, o, g, rain_kind=O.RAIN_STEP, rain=rain, rain_dt=3600.0)
    assert "forcing=uniform " in g.describe()
    o.advance(10 ** 6, t_end=200.0)
    g.advance(10 ** 6, t_end=200.0)
    storm = {"peak": 150.0, "x0": 0.0, "y0": 0.0, "vx": 1.5, "vy": 1.0, "sigma": 400.0}
    cells = np.array([12 * cols + 30, 40 * cols + 5], dtype=np.int32)
    q = np.array([[2.0, 1.0], [4.0, 0.5]])
    set_forcing(O, o, g, storm=storm, sources=cells, src_q=q, dtoq=400.0)
    assert "forcing=storm/sources " in g.describe()
    o.advance(10 ** 6, t_end=400.0)
    g.advance(10 ** 6, t_end=400.0)
    g.set_point_sources(np.zeros(0, dtype=np.int32), np.zeros((1, 0)), 1.0)
    set_forcing(O, o, g, rain_kind=O.RAIN_STEP, rain=rain, rain_dt=3600.0)
    assert "forcing=uniform " in g.describe()
    o.advance(10 ** 6, t_end=600.0)
    g.advance(10 ** 6, t_end=600.0)
    a, b = o.state()["h"], g.depth()
    print("max |dh| =", max_abs(a, b))
    assert max_abs(a, b) <= TOL_MM
    bo, bg = o.budget(), g.budget()
    assert bg["t"] == pytest.approx(600.0, abs=1e-9) and o.state()["t"] == pytest.approx(600.0, abs=1e-9)
    assert bg["source_in"] == pytest.approx(bo["source_in"], rel=1e-4)
    assert bg["rain_in"] == pytest.approx(bo["rain_in"], rel=1e-4)


def test_f32_dam_break_front(oracle_mod, sw2d_mod):
    """A frictionless dam break is a moving discontinuity: at the same
    simulated time (the CFL step of each run follows its own thin-film tip
    velocities, so step counts differ), FP32 and FP64 agree on volume, on the
    front position within one cell and in the mean depth error, before the
    wave reaches the downstream wall."""
    from sw2d import scenarios as S
    s = S.dam_break_channel(64, 512, 1.0, x_gate=128.0)
    o = oracle_mod.Oracle(64, 512, 1.0, 1.0, s["z"], dt_mode=1, dt=1.0)
    o.set_state(s["h0"])
    g = _f32(sw2d_mod, 64, 512, 1.0, s["z"], s["h0"], kernel=2, dt_mode=1, dt=1.0)
    o.advance(10 ** 6, t_end=4.0)
    g.advance(10 ** 6, t_end=4.0)
    assert abs(g.budget()["t"] - 4.0) < 1e-9 and abs(o.state()["t"] - 4.0) < 1e-9
    a, b = o.state()["h"], g.depth()
    front = lambda h: int(np.max(np.nonzero(h[32] > 1e-2)[0]))
    print("front", front(a), front(b), "mean |dh|", float(np.mean(np.abs(a - b))), "max", max_abs(a, b))
    assert front(a) < 500
    assert abs(front(a) - front(b)) <= 1
    assert float(np.mean(np.abs(a - b))) <= 5e-3
    assert g.budget()["volume"] == pytest.approx(o.volume(), rel=1e-6)


def test_compensated_depth_keeps_sub_ulp_rain(sw2d_mod):
    """A closed flat basin 1 m deep under rain of 0.01 mm/h: each step adds
    about 2.8e-9 m, below half an ulp of 1.0 in FP32 (6e-8).  The compensated
    depth must keep all of it: the volume gain equals the FP64 rain budget
    (a plain FP32 state would gain nothing)."""
    rows, cols = 64, 80
    z = np.zeros((rows, cols))
    h0 = np.ones((rows, cols))
    g = _f32(sw2d_mod, rows, cols, 10.0, z, h0, kernel=2, dt_mode=0, dt=0.5)
    g.set_rain(sw2d_mod.RAIN_STEP, [0.01], 1e6)
    assert g.advance(2000) == 2000
    b = g.budget()
    gain = b["volume"] - b["volume0"]
    assert b["rain_in"] > 0
    assert gain == pytest.approx(b["rain_in"], rel=1e-3)
    assert float(np.mean(g.depth() - 1.0)) == pytest.approx(b["rain_in"] / (rows * cols * 100.0), rel=1e-3)


def test_compensated_depth_in_the_batch(sw2d_mod):
    """The same through the batched kernel."""
    rows, cols = 64, 80
    bt = sw2d_mod.Batch(chunk=24, max_scenarios=4)
    cfg = sw2d_mod.default_config(rows=rows, cols=cols, dx=10.0, dy=10.0, precision=sw2d_mod.PREC_F32,
                                  dt_mode=sw2d_mod.DT_CFL, dt=0.5, cfl=0.5)
    sid = bt.add(cfg, np.zeros((rows, cols)), np.ones((rows, cols)), rain_kind=sw2d_mod.RAIN_STEP, rain=[0.01],
                 rain_dt=1e6, t_end=2000.0)
    running = 1
    while running:
        running = bt.advance(48)
    b = bt.budget(sid)
    assert b["rain_in"] > 0
    assert b["volume"] - b["volume0"] == pytest.approx(b["rain_in"], rel=1e-3)
    bt.close()
