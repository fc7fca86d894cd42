"""The large-domain comparison's statistics on the host (CPU): the pointwise
|FP64 - FP32| figures and the flooded-area difference reported against the
1 mm / 0.1 % bars, on a constructed case with known answers."""
import numpy as np
import pytest


def test_spread_known_answers():
    from sw2d import large_domain as L
    a = np.zeros((100, 100))
    a[:50] = 0.2                      # 5000 wet cells (> th = 1e-4)
    c = a.copy()
    c[0, :10] += 2e-3                 # 10 cells differ by 2 mm
    c[1, :5] += 5e-4                  # 5 cells by 0.5 mm
    c[99, 99] = 5e-5                  # one more cell, still dry (below th)
    c[98, 0] = 1e-3                   # one newly wet cell
    s = L.spread(a, c)
    assert s["max"] == pytest.approx(2e-3)
    assert s["cells_over_1mm"] == 10
    assert s["wet_cells"] == 5000
    assert s["flooded_area_rel_diff"] == pytest.approx(1 / 5000)
    assert s["p50"] == 0.0 and s["p99.99"] > s["p99"] >= 0.0


def test_storm_moves_along_the_diagonal_at_10_m_per_s():
    from sw2d import large_domain as L
    p = L.storm_params(8192, 2.0)
    assert np.hypot(p["vx"], p["vy"]) == pytest.approx(10.0) and p["vx"] == p["vy"] > 0
    assert p["peak"] == 80.0 and p["sigma"] == 2000.0
