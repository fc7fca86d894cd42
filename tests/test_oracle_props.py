"""Size-independent properties of the oracle (CPU): conservation, symmetry,
determinism across thread counts, the CFL rule, walls."""
import numpy as np
import pytest


def _dam(O, rows=32, cols=64, **kw):
    from sw2d import scenarios as S
    s = S.dam_break_channel(rows, cols, 1.0, x_gate=cols / 2)
    o = O.Oracle(rows, cols, 1.0, 1.0, s["z"], manning=kw.pop("manning", 0.0), dt_mode=1, dt=1.0, cfl=0.5, **kw)
    o.set_state(s["h0"])
    return o, s


def test_volume_conserved_with_walls(oracle_mod):
    o, s = _dam(oracle_mod)
    v0 = o.volume()
    o.advance(300)
    b = o.budget()
    assert abs(o.volume() + 0.0 - v0 - b["clamp_gain"]) / v0 < 1e-12


def test_row_symmetry(oracle_mod):
    """A 1D dam break stays identical across rows (walls north and south)."""
    o, s = _dam(oracle_mod)
    o.advance(200)
    h = o.state()["h"]
    assert np.array_equal(h, np.repeat(h[:1], h.shape[0], axis=0))


def test_thread_count_does_not_change_results(oracle_mod):
    o1, _ = _dam(oracle_mod, threads=1)
    o1.advance(50)
    h1 = o1.state()["h"]
    o2, _ = _dam(oracle_mod, threads=4)
    o2.advance(50)
    assert np.array_equal(h1, o2.state()["h"])
    oracle_mod.lib().orc_set_threads(oracle_mod.max_threads())


def test_cfl_rule_initial_step(oracle_mod):
    o, _ = _dam(oracle_mod)
    # dt2 = 0.5 * dx / sqrt(g h) with h = 10 at the still, wet faces
    assert o.next_dt() * 2 == pytest.approx(0.5 / np.sqrt(9.8 * 10.0), rel=1e-15)


def test_fixed_dt_time_accumulates_like_reference(oracle_mod):
    from sw2d import scenarios as S
    s = S.dam_break_channel(8, 16, 1.0, x_gate=8)
    o = oracle_mod.Oracle(8, 16, 1.0, 1.0, s["z"], dt_mode=0, dt=0.04)
    o.set_state(s["h0"])
    n = o.advance(10 ** 9, t_end=1.0)
    t = 0.0
    k = 0
    while t + 0.04 <= 1.0:  # cu:1256, time += dt twice (cu:1297, cu:1335)
        t = t + 0.04
        t = t + 0.04
        k += 1
    assert n == k and o.state()["t"] == t


def test_nan_depth_gives_nan_faces_in_the_oracle(oracle_mod):
    """The reference's arithmetic propagates a NaN depth into its faces (the
    GPU watchdog reports exactly this case)."""
    z = np.zeros((30, 40))
    h0 = np.full((30, 40), 0.5)
    h0[15, 20] = np.nan
    o = oracle_mod.Oracle(30, 40, 1.0, 1.0, z, dt_mode=0, dt=0.01)
    o.set_state(h0)
    o.advance(1, 1e9)
    st = o.state()
    assert np.isnan(st["um"]).any() or np.isnan(st["vn"]).any()


def test_lake_at_rest_stays_at_rest(oracle_mod):
    """A flat water surface over an uneven bed, every cell wet, with Manning
    friction: the surface-slope term vanishes and no dry-bed rule applies.
    On a bed of dyadic elevations (every sum exact) the state does not move
    at all.  On an arbitrary bed it moves only by FP64 rounding: the
    reference evaluates the slope as ((hb + zb) - ha) - za (cu:166), which
    rounds even when hb + zb == ha + za exactly."""
    O = oracle_mod
    rows, cols = 40, 56
    z = np.random.default_rng(3).uniform(0.0, 2.0, (rows, cols))
    for bed, tol in ((np.round(z * 64.0) / 64.0, 0.0), (z, 1e-12)):
        h0 = 3.0 - bed
        o = O.Oracle(rows, cols, 5.0, 5.0, bed, manning=0.03, dt_mode=0, dt=0.1)
        o.set_state(h0)
        o.advance(200, 1e9)
        st = o.state()
        assert np.max(np.abs(st["h"] - h0)) <= tol
        assert np.max(np.abs(st["um"])) <= 10 * tol and np.max(np.abs(st["vn"])) <= 10 * tol


def test_budget_closes_with_open_edge_rain_sources_evaporation(oracle_mod):
    """Stored volume = initial + rain + sources - evaporation - outflow through
    the open south edge + water created by the depth clamp, to FP64 rounding,
    on a run that uses every forcing at once."""
    from sw2d import scenarios as S
    O = oracle_mod
    rows, cols = 48, 40
    s = S.catchment(rows, dx=10.0, seed=6, cols=cols)
    o = O.Oracle(rows, cols, 10.0, 10.0, s["z"], n=s["n"], dt_mode=1, dt=1.0, cfl=0.5, south_open=1,
                 EV_WL_min=0.001, INT=0.1, INF=0.2, LWL=0.05)
    o.set_state(s["h0"])
    v0 = o.volume()
    cells = np.array([5 * cols + 7, 30 * cols + 20], dtype=np.int32)
    q = np.array([[1.0, 0.5], [2.0, 0.0], [0.5, 1.5]])
    o.set_forcing(O.OracleForcing(rain_kind=O.RAIN_LINEAR, rain=np.array([30.0, 90.0, 10.0]), rain_dt=300.0,
                                  ev=np.array([5e-7, 8e-7]), ev_dt=600.0, sources=cells, src_q=q, dtoq=300.0))
    o.advance(10 ** 6, t_end=900.0)
    b = o.budget()
    assert b["rain_in"] > 0 and b["source_in"] > 0 and b["evap_out"] > 0 and b["outflow"] > 0
    expect = v0 + b["rain_in"] + b["source_in"] - b["evap_out"] - b["outflow"] + b["clamp_gain"]
    assert abs(o.volume() - expect) <= 1e-9 * max(v0, 1.0)


def test_transposed_problem_gives_the_transposed_solution(oracle_mod):
    """The x-face (cu:116-225) and y-face (cu:232-342) updates are mirror
    images, including the column-0 / row-0 rules, so solving the transposed
    problem (rows <-> cols, dx <-> dy, um <-> vn) gives the transposed
    solution, bit for bit, here with dx != dy, per-cell n and rain.  An
    index slip in either direction breaks this."""
    from sw2d import scenarios as S
    O = oracle_mod
    s = S.catchment(36, dx=10.0, seed=4, cols=52)

    def run(z, n, h0, dx, dy):
        o = O.Oracle(z.shape[0], z.shape[1], dx, dy, z, n=n, dt_mode=0, dt=0.5)
        o.set_state(h0)
        o.set_forcing(O.OracleForcing(rain_kind=O.RAIN_STEP, rain=np.array([60.0]), rain_dt=3600.0))
        o.advance(400, 1e9)
        return o.state()

    a = run(s["z"], s["n"], s["h0"], 10.0, 8.0)
    b = run(s["z"].T.copy(), s["n"].T.copy(), s["h0"].T.copy(), 8.0, 10.0)
    assert np.array_equal(a["h"], b["h"].T)
    assert np.array_equal(a["um"], b["vn"].T) and np.array_equal(a["vn"], b["um"].T)
    assert a["h"].max() > s["h0"].max()  # the rain did something
