"""sw2d_volume_noalloc: the mass-balance volume sum for callers that cannot
allocate device memory (a host model whose memory pool already owns the
whole GPU, or one that must not call the allocator inside its time loop).
It keeps its partial sums in a fixed array inside the library instead of a
cudaMalloc'd buffer.

Checked through the C ABI against the existing entry point (sw2d_get_budget's
volume of the same state) and against a numpy sum of the same field, within
the test suite's FP64 budget tolerance, on two calls in a row; on a caller's
own stream; on a grid at the size limit; and after a larger call, whose
partial sums a smaller call must not pick up.  This file is named so that
pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # FP64 budget sums, different but deterministic summation orders


def _noalloc(sw2d, dev_depth, dev_mask, rows, cols, pitch, area, stream=None):
    out = C.c_double()
    st = sw2d.load().sw2d_volume_noalloc(C.c_void_p(dev_depth), C.c_void_p(dev_mask) if dev_mask else None,
                                         rows, cols, pitch, area, C.c_void_p(stream) if stream else None,
                                         C.byref(out))
    return st, out.value


def test_volume_noalloc_matches_budget_volume(sw2d_mod):
    import torch
    from sw2d import scenarios as S
    rows, cols, dx = 300, 257, 5.0
    s = S.catchment(rows, dx=dx, seed=21, cols=cols)
    z = s["z"].copy()
    z[np.random.default_rng(21).random(z.shape) < 0.05] = -9999.0
    g = sw2d_mod.Solver(rows=rows, cols=cols, dx=dx, dy=dx, precision=sw2d_mod.PREC_F64, dt_mode=sw2d_mod.DT_CFL,
                        dt=2.0, south_open=1)
    g.set_static(z, s["n"])
    g.set_state(np.where(z != -9999.0, 0.02, 0.7))  # inactive cells get depth 0 on upload
    g.set_rain(sw2d_mod.RAIN_STEP, [80.0], 3600.0)
    g.advance(60)
    expect = g.budget()["volume"]
    depth = g.depth()
    mask = (z != -9999.0).astype(np.uint8)
    pitch = cols + 7  # a padded layout, as a caller's own buffers may have
    d_depth = torch.zeros((rows, pitch), dtype=torch.float64, device="cuda")
    d_depth[:, :cols] = torch.from_numpy(depth).cuda()
    d_depth[:, cols:] = 123.0  # padding must not be summed
    d_mask = torch.zeros((rows, pitch), dtype=torch.uint8, device="cuda")
    d_mask[:, :cols] = torch.from_numpy(mask).cuda()
    torch.cuda.synchronize()
    plain = float(np.sum(depth[mask == 1], dtype=np.float64)) * dx * dx  # without the library
    assert plain == pytest.approx(expect, rel=REL_TOL)
    results = []
    for _ in range(2):  # two calls in a row share the scratch array
        st, v = _noalloc(sw2d_mod, d_depth.data_ptr(), d_mask.data_ptr(), rows, cols, pitch, dx * dx)
        assert st == 0
        assert v == pytest.approx(expect, rel=REL_TOL)
        assert v == pytest.approx(plain, rel=REL_TOL)
        results.append(v)
    assert results[0] == results[1]
    s = torch.cuda.Stream()  # a caller's own stream
    with torch.cuda.stream(s):
        st, v = _noalloc(sw2d_mod, d_depth.data_ptr(), d_mask.data_ptr(), rows, cols, pitch, dx * dx,
                         stream=s.cuda_stream)
    assert st == 0 and v == results[0]
    st, v_nomask = _noalloc(sw2d_mod, d_depth.data_ptr(), 0, rows, cols, pitch, dx * dx)
    assert st == 0 and v_nomask == pytest.approx(expect, rel=REL_TOL)  # inactive cells hold 0


def test_volume_noalloc_rejects_oversized_and_bad_args(sw2d_mod):
    L = sw2d_mod.load()
    out = C.c_double()
    big = 8192 * 8192 + 1
    # beyond SW2D_NOALLOC_MAX_CELLS: refused before any GPU work
    assert L.sw2d_volume_noalloc(C.c_void_p(16), None, big, 1, 1, 1.0, None, C.byref(out)) == 1
    assert L.sw2d_volume_noalloc(C.c_void_p(16), None, 8193, 8192, 8192, 1.0, None, C.byref(out)) == 1
    assert L.sw2d_volume_noalloc(None, None, 4, 4, 4, 1.0, None, C.byref(out)) == 1
    assert L.sw2d_volume_noalloc(C.c_void_p(16), None, 4, 4, 3, 1.0, None, C.byref(out)) == 1
    assert L.sw2d_volume_noalloc(C.c_void_p(16), None, 4, 4, 4, 0.0, None, C.byref(out)) == 1


def _kahan(x):
    s = c = 0.0
    for v in x:
        y = v - c
        t = s + y
        c = (t - s) - y
        s = t
    return s


def test_volume_noalloc_at_the_size_limit_then_smaller(sw2d_mod):
    """A grid of 8192 x 8192 cells (the last chunk index is 8191 and the
    total lands in the array's last slot), then a smaller grid: each equals a
    compensated sum of its own field, so the second call picked up nothing
    the first one left behind."""
    import torch
    rows = cols = 8192
    rng = np.random.default_rng(8)
    big = rng.random((rows, cols))
    d_big = torch.from_numpy(big).cuda()
    torch.cuda.synchronize()
    st, v = _noalloc(sw2d_mod, d_big.data_ptr(), 0, rows, cols, cols, 4.0)
    assert st == 0
    assert v == pytest.approx(float(np.sum(big, dtype=np.float64)) * 4.0, rel=REL_TOL)
    del d_big
    small = rng.random((37, 53))
    d_small = torch.from_numpy(small).cuda()
    torch.cuda.synchronize()
    for _ in range(2):
        st, v2 = _noalloc(sw2d_mod, d_small.data_ptr(), 0, 37, 53, 53, 1.0)
        assert st == 0
        assert v2 == pytest.approx(_kahan(small.ravel()), rel=REL_TOL)
