"""The oracle's deterministic log/exp/power (the same algorithm runs in the
FP64 device path) against the platform libm: error bounds, not bits."""
import ctypes as C

import numpy as np


def _vec(O, name, x):
    f = getattr(O.lib(), name)
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    out = np.empty_like(x)
    f(x.ctypes.data, x.size, out.ctypes.data)
    return out


def test_pow43_error_bound(oracle_mod):
    rng = np.random.default_rng(0)
    x = np.exp(rng.uniform(np.log(1e-4), np.log(1e4), 100000))
    x = np.concatenate([x, [1e-4, 1.0, 2.0, 0.5, 10.0, 1e4]])
    got = _vec(oracle_mod, "orc_pow43_vec", x)
    rel = np.abs(got / np.power(x, 1.3333330) - 1.0)
    assert rel.max() < 2e-15  # within ~8 ulp of libm


def test_exp_error_bound(oracle_mod):
    y = np.random.default_rng(1).uniform(-700.0, 700.0, 100000)
    got = _vec(oracle_mod, "orc_exp_vec", y)
    assert np.max(np.abs(got / np.exp(y) - 1.0)) < 1e-15
    edge = _vec(oracle_mod, "orc_exp_vec", np.array([0.0, -800.0, 1e-300]))
    assert edge[0] == 1.0 and edge[1] == 0.0 and edge[2] == 1.0
