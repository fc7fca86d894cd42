"""The evaporation series (the reference's gpu_evaporation_calc,
SW2D-GPU.cu:557-587): the oracle's numpy restatement against the
reference's own kernel (tests/golden/ref_evaporation.npz, made on a GPU by
tests/golden/make_ref_evaporation_golden.py), and the library's
sw2d_evaporation_series -- the one the reference-format driver uses --
against the restatement.  Host computations only: no GPU needed.

Bar: bit for bit against the reference built with --fmad=false (the same
operations in the same order, no contraction); within 4 ulp of the
reference as shipped (nvcc contracts multiply-adds there).
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_evaporation.npz")


def _cases():
    return [str(c) for c in np.load(GOLD)["cases"]] if os.path.exists(GOLD) else []


@pytest.mark.skipif(not os.path.exists(GOLD), reason="reference-kernel fixture not generated yet")
@pytest.mark.parametrize("name", _cases())
def test_restatement_matches_reference_kernel(oracle_mod, name):
    d = np.load(GOLD)
    g = lambda k: d[f"{name}__{k}"]
    e = oracle_mod.evaporation_series(g("T"), g("Rg"), float(g("albedo")), float(g("dtime")))
    assert np.array_equal(e, g("off"))
    on = g("on")
    assert np.all(np.abs(e - on) <= 4 * np.spacing(np.maximum(np.abs(on), 1e-300)))
    assert np.any(e == 0.0) and np.all(e >= 0.0)


@pytest.mark.skipif(not os.path.exists(GOLD), reason="reference-kernel fixture not generated yet")
@pytest.mark.parametrize("name", _cases())
def test_library_series_matches_reference_kernel(sw2d_mod, name):
    d = np.load(GOLD)
    g = lambda k: d[f"{name}__{k}"]
    e = sw2d_mod.evaporation_series(g("T"), g("Rg"), float(g("albedo")), float(g("dtime")))
    assert np.array_equal(e, g("off"))


def test_library_series_matches_restatement(sw2d_mod, oracle_mod):
    rng = np.random.default_rng(5)
    T = rng.uniform(-10.0, 50.0, 5000)
    Rg = rng.uniform(-200.0, 1500.0, 5000)
    for albedo, dtime in ((0.25, 3600.0), (0.07, 60.0), (0.0, 1.0)):
        a = sw2d_mod.evaporation_series(T, Rg, albedo, dtime)
        b = oracle_mod.evaporation_series(T, Rg, albedo, dtime)
        assert np.array_equal(a, b)


def test_library_series_refuses_bad_arguments(sw2d_mod):
    import ctypes as C
    L = sw2d_mod.load()
    x = np.zeros(3)
    p = x.ctypes.data_as(C.c_void_p)
    assert L.sw2d_evaporation_series(p, p, 3, 0.25, 0.0, p) == sw2d_mod.native.ERR_INVALID_ARG
    assert L.sw2d_evaporation_series(None, p, 3, 0.25, 60.0, p) == sw2d_mod.native.ERR_INVALID_ARG
    assert L.sw2d_evaporation_series(p, p, -1, 0.25, 60.0, p) == sw2d_mod.native.ERR_INVALID_ARG
    assert L.sw2d_evaporation_series(None, None, 0, 0.25, 60.0, None) == sw2d_mod.native.OK  # empty series
