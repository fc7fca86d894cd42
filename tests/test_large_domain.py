"""The large-single-domain configuration at reduced size: FP32 state with
FP64 budgets against the FP64 path under a moving Gaussian storm.  Bounds:
max |dh| <= 1 mm, flooded area within 0.1 %, relative volume error <= 1e-6."""
import pytest

pytestmark = pytest.mark.gpu


def test_large_domain_reduced(sw2d_mod):
    from sw2d import large_domain as L
    r = L.compare(size=768, dx=20.0, horizon=900.0, seed=5)
    print(r)
    assert r["f32"]["iterations"] > 50
    assert r["max_abs_dh_m"] <= 1e-3
    assert r["flooded_area_rel_diff"] <= 1e-3
    assert r["f32"]["volume_rel_error"] <= 1e-6
