"""The CPU oracle against the reference's shipped known-answer vector.

db/dam_break/output/Results_0.vtk is the first VTK the reference writes
(SW2D-GPU.cu:1339-1472): depth = initial condition, velocities after one
iteration, rows flipped (cu:1381), x_velocity = vv (cu:1436),
y_velocity = -uu (cu:1452), every value printed with "%f".
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "dam_break.npz")


def _fmt(a):
    return np.array([float("%f" % v) for v in np.ravel(a)])


def _dam_break_oracle(O, d, **kw):
    r, c = int(d["rows"]), int(d["cols"])
    o = O.Oracle(r, c, float(d["dx"]), float(d["dx"]), d["z"], nodata=float(d["nodata"]),
                 manning=float(d["manning"]), INT=float(d["INT"]), INF=float(d["INF"]),
                 LWL=float(d["LWL"]), EV_WL_min=float(d["EV_WL_min"]), dt_mode=0, dt=float(d["dt"]), **kw)
    o.set_state(d["h0"])
    return o


def test_results0_vtk_exact(oracle_mod):
    d = np.load(GOLD)
    o = _dam_break_oracle(oracle_mod, d)
    assert o.advance(1, 6000.0) == 1
    uu, vv = o.cell_velocity()
    assert np.array_equal(_fmt(-uu[::-1]), d["vtk_y_velocity"])
    assert np.array_equal(_fmt(vv[::-1]), d["vtk_x_velocity"])
    assert np.array_equal(_fmt(d["h0"][::-1]), d["vtk_depth"])
    assert np.array_equal(_fmt(d["z"][::-1]), d["vtk_elevation"])
    # the hand check: dry-bed rule 2 through the 11-cell breach (cu:149-158)
    st = o.state()
    assert st["um"][14, 44] == pytest.approx(0.35 * 5 * np.sqrt(2 * 9.8 * 5), rel=1e-15)
    assert np.count_nonzero(uu) == 22


def test_golden_has_22_velocities():
    d = np.load(GOLD)
    y = d["vtk_y_velocity"]
    assert np.count_nonzero(y) == 22 and np.all(y[y != 0] == -3.464823)


def test_planted_mistake_is_caught(oracle_mod):
    """A wrong constant planted in the oracle (g = 9.81 instead of the
    reference's 9.80, cu:809) must break the golden comparison."""
    d = np.load(GOLD)
    o = _dam_break_oracle(oracle_mod, d, g=9.81)
    o.advance(1, 6000.0)
    uu, _ = o.cell_velocity()
    assert not np.array_equal(_fmt(-uu[::-1]), d["vtk_y_velocity"])
