"""A lake at rest on the GPU: a flat water surface over a bed of dyadic
elevations (every sum and difference exact in FP32 and FP64), all cells wet,
Manning friction, fixed dt: the surface-slope term is exactly zero and no
dry-bed rule applies, so neither path may move the state at all."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_lake_at_rest_on_the_gpu(sw2d_mod, prec):
    rows, cols = 40, 70
    z = np.round(np.random.default_rng(3).uniform(0.0, 2.0, (rows, cols)) * 64.0) / 64.0
    h0 = 3.0 - z
    p = sw2d_mod.PREC_F64 if prec == "f64" else sw2d_mod.PREC_F32
    with sw2d_mod.Solver(rows=rows, cols=cols, dx=5.0, dy=5.0, precision=p, dt_mode=sw2d_mod.DT_FIXED, dt=0.1,
                         manning=0.03) as g:
        g.set_static(z)
        g.set_state(h0)
        assert g.advance(200, t_end=1e9) == 200
        st = g.state()
        assert np.array_equal(st["h"], h0)
        assert not np.any(st["um"]) and not np.any(st["vn"])
