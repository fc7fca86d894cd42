"""Randomised properties of the oracle (CPU): grid shapes, cell sizes, beds
and initial states drawn by hypothesis, a bounded number of small cases.

  * transposing the problem transposes the solution, bit for bit;
  * with walls all round and no forcing, volume + clamp gain is conserved;
  * a lake at rest over a dyadic bed does not move.
"""
import numpy as np
import pytest

hyp = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

SETTINGS = dict(max_examples=25, deadline=None, derandomize=True)


def _case(seed, rows, cols, wet_frac, holes):
    rng = np.random.default_rng(seed)
    z = rng.uniform(0.0, 1.5, (rows, cols))
    if holes:
        z[rng.random((rows, cols)) < 0.08] = -9999.0  # inactive cells
    h = rng.uniform(0.0, 0.8, (rows, cols)) * (rng.random((rows, cols)) < wet_frac)
    n = rng.uniform(0.0, 0.06, (rows, cols))
    return z, h, n


@settings(**SETTINGS)
@given(seed=st.integers(0, 10 ** 6), rows=st.integers(1, 24), cols=st.integers(1, 24),
       dx=st.sampled_from([0.5, 1.0, 2.0]), dy=st.sampled_from([0.5, 1.0, 3.0]),
       wet=st.floats(0.2, 1.0), holes=st.booleans())
def test_transposition_symmetry(oracle_mod, seed, rows, cols, dx, dy, wet, holes):
    O = oracle_mod
    z, h, n = _case(seed, rows, cols, wet, holes)

    def run(z, h, n, dx, dy):
        o = O.Oracle(z.shape[0], z.shape[1], dx, dy, z, n=n, dt_mode=0, dt=0.01)
        o.set_state(h)
        o.advance(60, 1e9)
        return o.state()

    a = run(z, h, n, dx, dy)
    b = run(z.T.copy(), h.T.copy(), n.T.copy(), dy, dx)
    assert np.array_equal(a["h"], b["h"].T)
    assert np.array_equal(a["um"], b["vn"].T) and np.array_equal(a["vn"], b["um"].T)


@settings(**SETTINGS)
@given(seed=st.integers(0, 10 ** 6), rows=st.integers(2, 28), cols=st.integers(2, 28),
       wet=st.floats(0.2, 1.0), holes=st.booleans(), cfl=st.booleans())
def test_volume_conserved_with_walls(oracle_mod, seed, rows, cols, wet, holes, cfl):
    O = oracle_mod
    z, h, n = _case(seed, rows, cols, wet, holes)
    o = O.Oracle(rows, cols, 1.0, 1.0, z, n=n, dt_mode=1 if cfl else 0, dt=0.01, cfl=0.5)
    o.set_state(h)
    v0 = o.volume()
    o.advance(80, 1e9)
    b = o.budget()
    assert abs(o.volume() - v0 - b["clamp_gain"]) <= 1e-12 * max(v0, 1.0)


@settings(**SETTINGS)
@given(seed=st.integers(0, 10 ** 6), rows=st.integers(1, 24), cols=st.integers(1, 24),
       level=st.sampled_from([2.0, 2.5, 4.0]))
def test_lake_at_rest_dyadic_bed(oracle_mod, seed, rows, cols, level):
    O = oracle_mod
    z = np.round(np.random.default_rng(seed).uniform(0.0, 1.9, (rows, cols)) * 32.0) / 32.0
    h0 = level - z
    o = O.Oracle(rows, cols, 2.0, 2.0, z, manning=0.04, dt_mode=0, dt=0.05)
    o.set_state(h0)
    o.advance(50, 1e9)
    s = o.state()
    assert np.array_equal(s["h"], h0) and not np.any(s["um"]) and not np.any(s["vn"])
