"""The reference's own CUDA kernels timed on this GPU beside our paths.

The harness replays the reference's loop as shipped (nine launches per
iteration, each followed by a device synchronisation, and the two host-to-
device copies of the point-source vector, SW2D-GPU.cu:1256-1336) on the
2048 x 2048 catchment with the reference's fixed time step; our FP64 and
FP32 paths run the same grid and dt.  Prints cell-updates/s for the three.
Asserted: the FP32 path at least 10x the reference's own FP64 kernels, and
the bit-reproducible FP64 path (no FMA, deterministic power function) in the
reference's speed class (measured on GB300: 1.13e9 against 1.12e9)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 2048
DT = 0.05


def test_reference_kernels_speed_against_ours(sw2d_mod):
    import ref_harness as R
    if not R.available("on"):
        pytest.skip("the reference's kernels were not built here")
    from sw2d import scenarios as S
    s = S.catchment(N, dx=5.0, seed=1, manning=0.03)
    h0 = np.full((N, N), 0.005)
    mod = R.RefModule("on")  # nvcc's default contraction, as shipped
    run = R.RefRun(mod, N, N, 5.0, s["z"], h0, 0.03, dt=DT, rain=[50.0 / 60.0] * 200, dtrain=60.0)
    run.run(2)
    mod.torch.cuda.synchronize()
    t0 = time.perf_counter()
    run.run(10)
    mod.torch.cuda.synchronize()
    ref_rate = N * N * 10 / (time.perf_counter() - t0)
    del run

    rates = {}
    for name, prec in (("fp64", sw2d_mod.PREC_F64), ("fp32", sw2d_mod.PREC_F32)):
        g = sw2d_mod.Solver(rows=N, cols=N, dx=5.0, dy=5.0, precision=prec, dt=DT, manning=0.03)
        g.set_static(s["z"])
        g.set_rain(sw2d_mod.RAIN_COMPAT, [50.0 / 60.0] * 200, 60.0)
        g.set_state(h0)
        g.advance(48)
        g.synchronize()
        t0 = time.perf_counter()
        n = g.advance(96 if name == "fp64" else 480)
        g.synchronize()
        rates[name] = N * N * n / (time.perf_counter() - t0)
        g.close()
    print(f"cell-updates/s on {N}x{N}: reference kernels as shipped {ref_rate:.3e}, "
          f"our FP64 {rates['fp64']:.3e} ({rates['fp64'] / ref_rate:.1f}x), "
          f"our FP32 {rates['fp32']:.3e} ({rates['fp32'] / ref_rate:.1f}x)")
    assert rates["fp32"] >= 10.0 * ref_rate
    assert rates["fp64"] >= 0.8 * ref_rate
