"""Checkpoint/restore and failure detection through the C ABI.

A restored handle continues bit for bit as the one the checkpoint was taken
from.  A non-finite value planted in the input state is reported as
SW2D_ERR_NONFINITE by the device-side watchdog (a status, never a GPU
fault)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver(sw2d, prec, s, **kw):
    g = sw2d.Solver(rows=80, cols=64, dx=5.0, dy=5.0, precision=prec, dt_mode=sw2d.DT_CFL, dt=2.0, south_open=1,
                    **kw)
    g.set_static(s["z"], s["n"])
    g.set_rain(sw2d.RAIN_STEP, [150.0], 3600.0)
    return g


@pytest.mark.parametrize("prec", [0, 1])
def test_restore_continues_bit_for_bit(sw2d_mod, prec):
    from sw2d import scenarios as S
    s = S.catchment(80, dx=5.0, seed=17, cols=64)
    a = _solver(sw2d_mod, prec, s)
    a.set_state(s["h0"])
    a.advance(100)
    ck = a.checkpoint()
    a.advance(77)
    b = _solver(sw2d_mod, prec, s)
    b.restore(ck)
    assert b.budget()["steps"] == 100
    b.advance(77)
    sa, sb = a.state(), b.state()
    for k in ("h", "um", "vn"):
        assert np.array_equal(sa[k], sb[k]), k
    ba, bb = a.budget(), b.budget()
    assert ba["t"] == bb["t"] and ba["steps"] == bb["steps"] == 177
    for k in ("rain_in", "outflow", "clamp_gain", "volume"):
        assert bb[k] == pytest.approx(ba[k], rel=1e-12, abs=1e-12)


def test_checkpoint_rejects_other_config(sw2d_mod):
    from sw2d import scenarios as S
    s = S.catchment(80, dx=5.0, seed=17, cols=64)
    a = _solver(sw2d_mod, 0, s)
    a.set_state(s["h0"])
    ck = a.checkpoint()
    b = _solver(sw2d_mod, 1, s)  # FP32: different layout
    with pytest.raises(sw2d_mod.SW2DError) as e:
        b.restore(ck)
    assert e.value.status == 1
    with pytest.raises(sw2d_mod.SW2DError):
        b.restore(b"not a checkpoint")


@pytest.mark.parametrize("prec", [0, 1])
def test_nonfinite_elevation_is_reported(sw2d_mod, prec):
    """A corrupt DEM value (NaN, not NODATA) inside a wet region makes the
    momentum update of its faces NaN; the watchdog turns that into
    SW2D_ERR_NONFINITE."""
    z = np.zeros((30, 40))
    z[15, 20] = np.nan
    h0 = np.full((30, 40), 0.5)
    g = sw2d_mod.Solver(rows=30, cols=40, dx=1.0, dy=1.0, precision=prec, dt_mode=sw2d_mod.DT_FIXED, dt=0.01)
    g.set_static(z)
    g.set_state(h0)
    with pytest.raises(sw2d_mod.SW2DError) as e:
        g.advance(50, 1e9)
    assert e.value.status == 4  # SW2D_ERR_NONFINITE
    assert g.budget()["nonfinite"] == 1


@pytest.mark.parametrize("prec", [0, 1])
def test_nonfinite_depth_is_reported(sw2d_mod, prec):
    """A NaN depth makes the momentum update of its faces NaN, as in the
    reference's arithmetic (its dry-bed product test and friction guard are
    false for NaN, cu:149, cu:197); the watchdog reports it."""
    z = np.zeros((30, 40))
    h0 = np.full((30, 40), 0.5)
    h0[15, 20] = np.nan
    g = sw2d_mod.Solver(rows=30, cols=40, dx=1.0, dy=1.0, precision=prec, dt_mode=sw2d_mod.DT_FIXED, dt=0.01)
    g.set_static(z)
    g.set_state(h0)
    with pytest.raises(sw2d_mod.SW2DError) as e:
        g.advance(20, 1e9)
    assert e.value.status == 4  # SW2D_ERR_NONFINITE
