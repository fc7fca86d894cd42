"""The CPU oracle against outputs of the reference's own CUDA kernels
(tests/golden/ref_kernels.npz, made by tests/golden/make_ref_golden.py on a
GPU from device-only builds of the unmodified reference source).

"off": reference built with --fmad=false.  Without friction the update uses
only + - * / sqrt and must agree to the bit; with friction the reference
calls CUDA's pow while the oracle uses its own power function (a few ulp
apart), so depths must agree within 1e-9 m with identical wet/dry masks.
"on": the reference as shipped (nvcc FMA contraction): within 1e-9 m.
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.npz")
TH = 1.0e-4

pytestmark = pytest.mark.skipif(not os.path.exists(GOLD), reason="reference-kernel fixture not generated yet")


def _cases():
    if not os.path.exists(GOLD):
        return []
    return [str(c) for c in np.load(GOLD)["cases"]]


def _run_oracle(O, d, name):
    g = lambda k, default=None: d[f"{name}__{k}"] if f"{name}__{k}" in d.files else default
    rows, cols = int(g("rows")), int(g("cols"))
    dx = float(g("dx"))
    kw = {k: float(g(k)) for k in ("INT", "INF", "LWL", "EV_WL_min") if g(k) is not None}
    o = O.Oracle(rows, cols, dx, dx, g("z"), manning=float(g("manning")), dt_mode=0, dt=float(g("dt")), **kw)
    o.set_state(g("h0"))
    f = {}
    if g("rain") is not None:
        f.update(rain_kind=O.RAIN_COMPAT, rain=g("rain"), rain_dt=float(g("dtrain")))
    if g("sources") is not None:
        src = np.asarray(g("sources"))
        keep = src < rows * cols  # the reference writes sources past the grid into its padding row
        q = np.asarray(g("q")).reshape(-1, src.size)
        f.update(sources=src[keep], src_q=q[:, keep], dtoq=float(g("dtoq")))
    o.set_forcing(O.OracleForcing(**f))
    n = int(g("steps"))
    assert o.advance(n, 1e12) == n
    return o, g


@pytest.mark.parametrize("name", _cases())
def test_oracle_matches_reference_kernels(oracle_mod, name):
    d = np.load(GOLD)
    o, g = _run_oracle(oracle_mod, d, name)
    st = o.state()
    assert st["t"] == float(g("off_t"))
    ref = g("off_h")
    if float(g("manning")) == 0.0:
        assert np.array_equal(st["h"], ref), np.max(np.abs(st["h"] - ref))
        assert np.array_equal(st["um"], g("off_um"))
        assert np.array_equal(st["vn"], g("off_vn"))
        uu, vv = o.cell_velocity()
        assert np.array_equal(uu, g("off_uu")) and np.array_equal(vv, g("off_vv"))
    else:
        assert np.max(np.abs(st["h"] - ref)) <= 1e-9
        assert np.array_equal(st["h"] > TH, ref > TH)
    on = g("on_h")
    assert np.max(np.abs(st["h"] - on)) <= 1e-9
    assert np.array_equal(st["h"] > TH, on > TH)
