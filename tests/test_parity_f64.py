"""FP64 GPU path against the CPU oracle, through the C ABI.

Bar: bit-identical depth and discharges wherever the update involves only
+ - * / sqrt (no Manning friction power, no storm exponential), and within
1e-9 m otherwise (pow/exp differ by ulps between CUDA and glibc), with
identical wet/dry masks (h > th).
"""
import os

import numpy as np
import pytest

from helpers import make_pair, max_abs, same, set_forcing

pytestmark = pytest.mark.gpu

TOL_H = 1e-9   # m, FP64 mode
TH = 1.0e-4
GOLD = os.path.join(os.path.dirname(__file__), "golden", "dam_break.npz")


def _check_bitwise(o, g):
    a, b = o.state(), g.state()
    assert same(a["h"], b["h"]), max_abs(a["h"], b["h"])
    assert same(a["um"], b["um"]), max_abs(a["um"], b["um"])
    assert same(a["vn"], b["vn"]), max_abs(a["vn"], b["vn"])
    bud = g.budget()
    assert bud["t"] == a["t"] and bud["steps"] == a["steps"]


def _check_tol(o, g, tol=TOL_H):
    a, b = o.state(), g.state()
    assert max_abs(a["h"], b["h"]) <= tol
    assert np.array_equal(a["h"] > TH, b["h"] > TH)
    bud = g.budget()
    assert bud["steps"] == a["steps"]
    assert abs(bud["t"] - a["t"]) <= 1e-9 * max(1.0, abs(a["t"]))


def test_dam_break_channel_bitwise(oracle_mod, sw2d_mod):
    from sw2d import scenarios as S
    s = S.dam_break_channel(64, 128, 1.0, x_gate=64.0)
    o, g = make_pair(oracle_mod, sw2d_mod, 64, 128, 1.0, s["z"], s["h0"], dt_mode=1, dt=1.0, cfl=0.5)
    assert o.advance(300) == 300
    assert g.advance(300) == 300
    _check_bitwise(o, g)


def test_chunking_invariance(oracle_mod, sw2d_mod):
    """advance(a) + advance(b) == advance(a+b), for chunk sizes around the
    graph length."""
    from sw2d import scenarios as S
    s = S.dam_break_channel(40, 72, 1.0, x_gate=30.0)
    o, g = make_pair(oracle_mod, sw2d_mod, 40, 72, 1.0, s["z"], s["h0"])
    tot = 0
    for n in (1, 2, 47, 48, 49, 100, 5):
        assert g.advance(n) == n
        tot += n
    assert o.advance(tot) == tot
    _check_bitwise(o, g)


def test_cfl_run_ends_on_t_end(oracle_mod, sw2d_mod):
    from sw2d import scenarios as S
    s = S.dam_break_channel(16, 48, 1.0, x_gate=20.0)
    o, g = make_pair(oracle_mod, sw2d_mod, 16, 48, 1.0, s["z"], s["h0"])
    n_o = o.advance(10 ** 6, t_end=3.0)
    n_g = g.advance(10 ** 6, t_end=3.0)
    assert n_o == n_g > 0
    _check_bitwise(o, g)
    assert abs(g.budget()["t"] - 3.0) < 1e-9
    assert g.advance(10, t_end=3.0) == 0


def test_reference_dam_break_golden_through_abi(oracle_mod, sw2d_mod):
    """The reference's shipped Results_0.vtk reproduced by the GPU path."""
    d = np.load(GOLD)
    r, c = int(d["rows"]), int(d["cols"])
    g = sw2d_mod.Solver(rows=r, cols=c, dx=float(d["dx"]), dy=float(d["dx"]), nodata=float(d["nodata"]),
                        manning=float(d["manning"]), INT=float(d["INT"]), INF=float(d["INF"]), LWL=float(d["LWL"]),
                        EV_WL_min=float(d["EV_WL_min"]), precision=0, dt_mode=0, dt=float(d["dt"]))
    g.set_static(d["z"])
    g.set_state(d["h0"])
    assert g.advance(1, 6000.0) == 1
    fmt = lambda a: np.array([float("%f" % v) for v in np.ravel(a)])
    uu = g.field(sw2d_mod.FIELD_UU)
    vv = g.field(sw2d_mod.FIELD_VV)
    assert np.array_equal(fmt(-uu[::-1]), d["vtk_y_velocity"])
    assert np.array_equal(fmt(vv[::-1]), d["vtk_x_velocity"])
    assert np.array_equal(fmt(g.field(sw2d_mod.FIELD_ELEVATION)[::-1]), d["vtk_elevation"])


def test_reference_dam_break_200_steps(oracle_mod, sw2d_mod):
    """dam_break with the reference's friction (n = 0.012, pow): within 1e-9."""
    d = np.load(GOLD)
    r, c = int(d["rows"]), int(d["cols"])
    o, g = make_pair(oracle_mod, sw2d_mod, r, c, float(d["dx"]), d["z"], d["h0"], manning=float(d["manning"]),
                     dt_mode=0, dt=float(d["dt"]), INT=float(d["INT"]), INF=float(d["INF"]), LWL=float(d["LWL"]),
                     EV_WL_min=float(d["EV_WL_min"]))
    assert o.advance(200, 6000.0) == 200
    assert g.advance(200, 6000.0) == 200
    _check_tol(o, g)


def _catchment_case(oracle_mod, sw2d_mod, rows=72, cols=56, seed=3, holes=True, south_open=1, precision=0,
                    tile=None):
    from sw2d import scenarios as S
    s = S.catchment(rows, dx=5.0, seed=seed, cols=cols)
    z = s["z"].copy()
    if holes:  # NODATA islands and a NODATA border strip
        rng = np.random.default_rng(seed)
        z[rng.random(z.shape) < 0.03] = -9999.0
        z[:, :2] = -9999.0
    o, g = make_pair(oracle_mod, sw2d_mod, rows, cols, 5.0, z, s["h0"], n=s["n"], precision=precision,
                     south_open=south_open, dt_mode=1, dt=2.0, cfl=0.5, tile=tile)
    set_forcing(oracle_mod, o, g, rain_kind=2, rain=np.array([400.0, 120.0]), rain_dt=60.0)
    return o, g


def test_catchment_rain_masks_open_outflow(oracle_mod, sw2d_mod):
    o, g = _catchment_case(oracle_mod, sw2d_mod)
    assert o.advance(400) == 400
    assert g.advance(400) == 400
    _check_tol(o, g)
    bo, bg = o.budget(), g.budget()
    for k in ("rain_in", "outflow", "clamp_gain"):
        assert bg[k] == pytest.approx(bo[k], rel=1e-9, abs=1e-9)
    assert bg["outflow"] > 0


def test_catchment_f64_alt_tile(oracle_mod, sw2d_mod):
    o, g = _catchment_case(oracle_mod, sw2d_mod, rows=50, cols=70, seed=5, tile=(8, 32))
    o.advance(200)
    g.advance(200)
    _check_tol(o, g)


def test_compat_forcing_sources_evaporation(oracle_mod, sw2d_mod):
    """The reference's own forcing formulas: rain in mm per interval with its
    division quirk (cu:547-554), point sources incl. a sink (cu:532-546) with
    two sources on one cell (the later wins), evaporation (cu:589-601), the
    runoff fractions INT/INF/LWL (cu:627-634) and a fixed dt."""
    from sw2d import scenarios as S
    rows, cols = 40, 48
    s = S.catchment(rows, dx=10.0, seed=7, cols=cols, manning=0.03)
    h0 = np.where(s["z"] < np.percentile(s["z"], 20), 0.3, 0.0)
    o, g = make_pair(oracle_mod, sw2d_mod, rows, cols, 10.0, s["z"], h0, manning=0.03, dt_mode=0, dt=0.05,
                     INT=0.45, INF=0.20, LWL=0.30, EV_WL_min=0.05)
    rain = np.array([0.0, 3.0, 6.0, 1.0, 0.0, 2.0])
    ev = np.array([0.1, 0.2, 0.3, 0.2, 0.1, 0.0])
    cells = np.array([5 * cols + 7, 20 * cols + 30, 20 * cols + 30, 33 * cols + 3], dtype=np.int32)
    q = np.array([[0.5, 1.0, 2.0, -0.12], [1.5, 0.0, 3.0, -0.12], [0.2, 0.5, 1.0, -0.12],
                  [0.0, 0.0, 0.0, -0.12]])
    set_forcing(oracle_mod, o, g, rain_kind=1, rain=rain, rain_dt=3.0, ev=ev, ev_dt=3.0, sources=cells, src_q=q,
                dtoq=4.0)
    assert o.advance(150, 1e9) == 150
    assert g.advance(150, 1e9) == 150
    _check_tol(o, g)
    bo, bg = o.budget(), g.budget()
    for k in ("rain_in", "source_in", "evap_out"):
        assert bg[k] == pytest.approx(bo[k], rel=1e-9, abs=1e-9)


def test_storm_rain(oracle_mod, sw2d_mod):
    from sw2d import scenarios as S
    rows, cols = 48, 48
    s = S.catchment(rows, dx=20.0, seed=11, manning=0.05)
    o, g = make_pair(oracle_mod, sw2d_mod, rows, cols, 20.0, s["z"], s["h0"], manning=0.05, south_open=1,
                     dt_mode=1, dt=5.0)
    storm = {"peak": 300.0, "x0": 0.0, "y0": 0.0, "vx": 2.0, "vy": 2.0, "sigma": 300.0}
    set_forcing(oracle_mod, o, g, storm=storm)
    o.advance(300)
    g.advance(300)
    _check_tol(o, g)


@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (9, 1), (17, 33), (33, 17), (3, 65)])
def test_ragged_and_tiny_grids(oracle_mod, sw2d_mod, shape):
    rows, cols = shape
    rng = np.random.default_rng(rows * 100 + cols)
    z = rng.uniform(0, 0.5, (rows, cols))
    h0 = rng.uniform(0, 1.0, (rows, cols)) * (rng.random((rows, cols)) < 0.6)
    o, g = make_pair(oracle_mod, sw2d_mod, rows, cols, 1.0, z, h0, dt_mode=1, dt=0.5)
    o.advance(60)
    g.advance(60)
    _check_bitwise(o, g)


def test_all_nodata_grid(oracle_mod, sw2d_mod):
    z = np.full((20, 30), -9999.0)
    h0 = np.ones((20, 30))
    o, g = make_pair(oracle_mod, sw2d_mod, 20, 30, 1.0, z, h0, dt_mode=0, dt=0.1)
    assert g.advance(10, 1e9) == 10
    assert np.all(g.depth() == 0)
    assert g.budget()["volume"] == 0.0


def test_nonzero_initial_discharge(oracle_mod, sw2d_mod):
    """A state with discharges (um, vn) given, as a restart would supply."""
    rows, cols = 24, 40
    rng = np.random.default_rng(2)
    z = rng.uniform(0, 0.2, (rows, cols))
    h0 = 0.5 + rng.uniform(0, 0.5, (rows, cols))
    um = rng.uniform(-0.1, 0.1, (rows + 1, cols))
    vn = rng.uniform(-0.1, 0.1, (rows, cols + 1))
    um[0] = um[-1] = 0
    vn[:, 0] = vn[:, -1] = 0
    o, g = make_pair(oracle_mod, sw2d_mod, rows, cols, 1.0, z, h0)
    o.set_state(h0, um, vn)
    g.set_state(h0, um, vn)
    o.advance(100)
    g.advance(100)
    _check_bitwise(o, g)


def test_probe_and_fields(oracle_mod, sw2d_mod):
    from sw2d import scenarios as S
    s = S.dam_break_channel(16, 32, 1.0, x_gate=16.0)
    o, g = make_pair(oracle_mod, sw2d_mod, 16, 32, 1.0, s["z"], s["h0"])
    o.advance(40)
    g.advance(40)
    h = o.state()["h"]
    cells = np.array([0, 5, 16 * 32 - 1, 7 * 32 + 13], dtype=np.int32)
    assert np.array_equal(g.probe(cells), h.ravel()[cells])
    for bad in (-1, 16 * 32):  # outside the grid: refused on the host
        with pytest.raises(sw2d_mod.SW2DError) as e:
            g.probe(np.array([3, bad], dtype=np.int32))
        assert e.value.status == sw2d_mod.native.ERR_INVALID_ARG
    uu, vv = o.cell_velocity()
    assert same(g.field(sw2d_mod.FIELD_UU), uu)
    assert same(g.field(sw2d_mod.FIELD_VV), vv)


REF = os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.npz")


def _ref_cases():
    return [str(c) for c in np.load(REF)["cases"]] if os.path.exists(REF) else []


@pytest.mark.parametrize("name", _ref_cases())
def test_f64_path_matches_reference_kernels(sw2d_mod, name):
    """The FP64 GPU path against outputs of the reference's own CUDA kernels
    (fixture made by tests/golden/make_ref_golden.py): bit for bit without
    friction, within 1e-9 m and identical wet/dry masks with it."""
    d = np.load(REF)
    g = lambda k: d[f"{name}__{k}"] if f"{name}__{k}" in d.files else None
    rows, cols, dx = int(g("rows")), int(g("cols")), float(g("dx"))
    kw = {k: float(g(k)) for k in ("INT", "INF", "LWL", "EV_WL_min") if g(k) is not None}
    s = sw2d_mod.Solver(rows=rows, cols=cols, dx=dx, dy=dx, manning=float(g("manning")), precision=0, dt_mode=0,
                        dt=float(g("dt")), **kw)
    s.set_static(g("z"))
    s.set_state(g("h0"))
    if g("rain") is not None:
        s.set_rain(sw2d_mod.RAIN_COMPAT, g("rain"), float(g("dtrain")))
    if g("sources") is not None:
        src = np.asarray(g("sources"))
        keep = src < rows * cols
        q = np.asarray(g("q")).reshape(-1, src.size)
        s.set_point_sources(src[keep], q[:, keep], float(g("dtoq")))
    n = int(g("steps"))
    assert s.advance(n, 1e12) == n
    st = s.state()
    assert s.budget()["t"] == float(g("off_t"))
    if float(g("manning")) == 0.0:
        assert same(st["h"], g("off_h")) and same(st["um"], g("off_um")) and same(st["vn"], g("off_vn"))
        assert same(s.field(sw2d_mod.FIELD_UU), g("off_uu")) and same(s.field(sw2d_mod.FIELD_VV), g("off_vv"))
    else:
        assert max_abs(st["h"], g("off_h")) <= TOL_H
        assert np.array_equal(st["h"] > TH, g("off_h") > TH)
    assert max_abs(st["h"], g("on_h")) <= TOL_H
