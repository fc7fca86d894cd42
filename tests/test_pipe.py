"""Several iterations per launch (steps_per_launch, FP32 streaming kernel,
fixed time step): every warp keeps one unit for K iterations and waits only
for the units around it.  Through the C ABI, against the same kernel run one
launch per iteration: the state (depth, remainder, discharges), the time and
the step count are bit for bit the same; the FP64 budgets are the same terms
summed in another order (relative 1e-12).  Also against the FP64 oracle
within the FP32 bound, and the configurations the library refuses.
"""
import numpy as np
import pytest

from helpers import make_pair, max_abs, set_forcing

pytestmark = pytest.mark.gpu

TOL_MM = 1.0e-3
BUDGET_KEYS = ("rain_in", "source_in", "evap_out", "outflow", "clamp_gain")


def _solver(sw2d, rows, cols, dx, z, h0, n=None, spl=0, **kw):
    kw.setdefault("dt_mode", sw2d.DT_FIXED)
    g = sw2d.Solver(rows=rows, cols=cols, dx=dx, dy=dx, precision=sw2d.PREC_F32, kernel=sw2d.KERNEL_STREAM,
                    steps_per_launch=spl, **kw)
    g.set_static(z, n)
    g.set_state(h0)
    return g


def _catchment(rows, cols, seed, holes=True):
    from sw2d import scenarios as S
    s = S.catchment(rows, dx=5.0, seed=seed, cols=cols)
    z = s["z"].copy()
    if holes:
        z[np.random.default_rng(seed).random(z.shape) < 0.02] = -9999.0
    return s, z


def _same(a, b, budgets=True):
    ga, gb = a.state(), b.state()
    assert np.array_equal(a.depth(), b.depth())
    assert np.array_equal(ga["um"], gb["um"]) and np.array_equal(ga["vn"], gb["vn"])
    ba, bb = a.budget(), b.budget()
    assert ba["t"] == bb["t"] and ba["steps"] == bb["steps"]
    assert ba["volume"] == bb["volume"]
    if budgets:
        for k in BUDGET_KEYS:
            assert bb[k] == pytest.approx(ba[k], rel=1e-12, abs=1e-9), k


def _run(g, chunks):
    done = 0
    for c in chunks:
        done += g.advance(c)
    return done


@pytest.mark.parametrize("spl", [0, 7, 48, 100])
def test_pipe_uniform_forcing_matches_one_launch_per_iteration(sw2d_mod, spl):
    """Per-cell n, NODATA holes, step rain with runoff fractions and
    evaporation, open south edge; advances that stop inside a launch's
    iterations (150 = 3 x 48 + 6, and 37)."""
    rows, cols = 150, 170
    s, z = _catchment(rows, cols, 31)
    out = []
    for k in (1, spl):
        g = _solver(sw2d_mod, rows, cols, 5.0, z, s["h0"], n=s["n"], spl=k, dt=0.4, south_open=1,
                    INT=0.2, INF=0.1, LWL=0.01, EV_WL_min=0.002)
        g.set_rain(sw2d_mod.RAIN_STEP, [120.0, 30.0], 300.0)
        g.set_evaporation([2.0e-7], 3600.0)
        d = g.describe()
        assert ("stream_pipe_kernel" in d) == (k != 1)
        assert f"steps_per_launch={48 if k == 0 else k}" in d
        assert _run(g, (150, 37)) == 187
        out.append(g)
    _same(*out)
    # the pipelined handle issues two kernels per launch, and one plan kernel per advance
    assert out[1].launch_count() == 2 * sum(-(-c // (48 if spl == 0 else spl)) for c in (150, 37)) + 2
    for g in out:
        g.close()


def test_pipe_storm_sources_rain_weights(sw2d_mod):
    """The forms with the moving storm and point sources, and with per-cell
    rain factors, scalar n."""
    rows, cols = 120, 200
    s, z = _catchment(rows, cols, 32)
    cells = np.array([10 * cols + 40, 60 * cols + 150, 60 * cols + 150, 119 * cols + 3], dtype=np.int32)
    q = np.array([[1.0, 2.0, 0.5, 0.1], [3.0, 0.0, 1.0, 0.2], [0.5, 0.5, 0.5, 0.5]])
    w = np.random.default_rng(5).uniform(0.2, 1.8, (rows, cols))
    for form in ("storm_sources", "weights"):
        out = []
        for k in (1, 16):
            g = _solver(sw2d_mod, rows, cols, 5.0, z, s["h0"], spl=k, dt=0.4, south_open=1, manning=0.05)
            if form == "storm_sources":
                g.set_storm(150.0, 0.0, 0.0, 2.0, 1.0, 400.0)
                g.set_point_sources(cells, q, 60.0)
            else:
                g.set_rain(sw2d_mod.RAIN_LINEAR, [0.0, 90.0, 20.0], 120.0)
                g.set_rain_weights(w)
            assert _run(g, (100, 21)) == 121
            out.append(g)
        _same(*out)
        for g in out:
            g.close()


def test_pipe_stops_at_t_end(sw2d_mod):
    """A run bounded by t_end, not by a step count: the launch that reaches
    t_end runs only the iterations whose t + dt <= t_end (cu:1256)."""
    rows, cols = 64, 90
    s, z = _catchment(rows, cols, 33, holes=False)
    out = []
    for k in (1, 48):
        g = _solver(sw2d_mod, rows, cols, 5.0, z, s["h0"], n=s["n"], spl=k, dt=0.3)
        g.set_rain(sw2d_mod.RAIN_STEP, [80.0], 3600.0)
        n = g.advance(10 ** 6, t_end=31.7)
        out.append((g, n))
    (a, na), (b, nb) = out
    t, expect = 0.0, 0
    while t + 0.3 <= 31.7:  # the reference's loop condition, the same FP64 recurrence
        t = (t + 0.3) + 0.3
        expect += 1
    assert na == nb == expect and expect > 48
    _same(a, b)
    assert b.advance(10, t_end=31.7) == 0
    a.close()
    b.close()


def test_pipe_vs_oracle(oracle_mod, sw2d_mod):
    """The pipelined FP32 path against the FP64 oracle: max |dh| <= 1 mm,
    flooded area within 0.1 %, budget closure <= 1e-6."""
    rows, cols = 96, 80
    s, z = _catchment(rows, cols, 34)
    o, g64 = make_pair(oracle_mod, sw2d_mod, rows, cols, 5.0, z, s["h0"], n=s["n"], south_open=1, dt_mode=0,
                       dt=0.4)
    g64.close()
    g = _solver(sw2d_mod, rows, cols, 5.0, z, s["h0"], n=s["n"], spl=0, dt=0.4, south_open=1)
    set_forcing(oracle_mod, o, g, rain_kind=2, rain=np.array([100.0, 50.0]), rain_dt=300.0)
    assert o.advance(600) == 600
    assert g.advance(600) == 600
    a, b = o.state()["h"], g.depth()
    assert max_abs(a, b) <= TOL_MM
    na, nb = np.count_nonzero(a > 1e-4), np.count_nonzero(b > 1e-4)
    assert abs(na - nb) <= 1e-3 * max(na, 1)
    bud = g.budget()
    rhs = bud["volume0"] + bud["rain_in"] + bud["source_in"] - bud["evap_out"] - bud["outflow"] + bud["clamp_gain"]
    assert abs(bud["volume"] - rhs) <= 1e-6 * bud["volume"]
    g.close()


def test_pipe_checkpoint_restore_continues(sw2d_mod):
    """A pipelined run restored from a checkpoint continues bit for bit."""
    rows, cols = 70, 110
    s, z = _catchment(rows, cols, 35)
    a = _solver(sw2d_mod, rows, cols, 5.0, z, s["h0"], n=s["n"], spl=0, dt=0.4)
    a.set_rain(sw2d_mod.RAIN_STEP, [150.0], 3600.0)
    a.advance(60)
    ck = a.checkpoint()
    a.advance(70)
    b = _solver(sw2d_mod, rows, cols, 5.0, z, s["h0"], n=s["n"], spl=0, dt=0.4)
    b.set_rain(sw2d_mod.RAIN_STEP, [150.0], 3600.0)
    b.restore(ck)
    b.advance(70)
    assert np.array_equal(a.depth(), b.depth())
    assert a.budget()["t"] == b.budget()["t"]
    a.close()
    b.close()


def test_pipe_refused_configurations(sw2d_mod):
    import sw2d
    z = np.zeros((40, 40))
    for kw in (dict(dt_mode=sw2d.DT_CFL, cfl=0.5), dict(precision=sw2d.PREC_F64), dict(kernel=sw2d.KERNEL_TILE)):
        args = dict(rows=40, cols=40, dx=1.0, dy=1.0, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_FIXED, dt=0.01,
                    steps_per_launch=8)
        args.update(kw)
        with pytest.raises(sw2d.SW2DError):
            sw2d.Solver(**args)
    with pytest.raises(sw2d.SW2DError):  # more than 1024 iterations per launch
        sw2d.Solver(rows=40, cols=40, dx=1.0, dy=1.0, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_FIXED, dt=0.01,
                    steps_per_launch=1025)
    with pytest.raises(sw2d.SW2DError):  # strips shorter than the neighbour set allows
        sw2d.Solver(rows=40, cols=40, dx=1.0, dy=1.0, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_FIXED, dt=0.01,
                    steps_per_launch=8, strip_h=4)
    # the library's choice falls back to one launch per iteration instead
    with sw2d.Solver(rows=40, cols=40, dx=1.0, dy=1.0, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_FIXED, dt=0.01,
                     strip_h=4) as g:
        assert "steps_per_launch=1" in g.describe()
    with sw2d.Solver(rows=40, cols=40, dx=1.0, dy=1.0, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_CFL, dt=0.01) as g:
        g.set_static(z)
        assert "steps_per_launch=1" in g.describe()


def test_library_choice_of_steps_per_launch(sw2d_mod):
    """steps_per_launch = 0: several iterations per launch where one wave
    holds the grid in strips of at most 32 rows, one launch per iteration on
    a 2048^2 grid (52-row strips), and one launch per iteration while a storm
    or point sources are set (the form that carries them spills in the
    pipelined kernel) unless the caller asked for several; the results are
    the same bits either way."""
    import sw2d
    for n, expect in ((512, "steps_per_launch=48"), (2048, "steps_per_launch=1")):
        with sw2d.Solver(rows=n, cols=n, dx=5.0, dy=5.0, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_FIXED, dt=0.4,
                         kernel=sw2d.KERNEL_STREAM) as g:
            assert expect in g.describe(), g.describe()
    rows, cols = 120, 200
    s, z = _catchment(rows, cols, 43)
    out = []
    for k in (0, 16):
        g = _solver(sw2d_mod, rows, cols, 5.0, z, s["h0"], spl=k, dt=0.4, south_open=1, manning=0.05)
        assert "stream_pipe_kernel" in g.describe()
        g.set_storm(150.0, 0.0, 0.0, 2.0, 1.0, 400.0)
        d = g.describe()
        assert ("stream_pipe_kernel" in d) == (k == 16), d
        assert g.advance(100) == 100
        out.append(g)
    _same(*out)
    for g in out:
        g.close()
