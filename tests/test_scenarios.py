"""The seeded synthetic inputs of the benchmark configurations (CPU): they are
deterministic, have the documented structure, and the ensemble and request
stream follow their stated distributions."""
import builtins

import numpy as np
import pytest


def test_catchment_is_deterministic_and_seeded():
    from sw2d import scenarios as S
    a, b, c = S.catchment(96, seed=4), S.catchment(96, seed=4), S.catchment(96, seed=5)
    assert np.array_equal(a["z"], b["z"]) and np.array_equal(a["n"], b["n"])
    assert not np.array_equal(a["z"], c["z"])
    r = S.catchment(40, seed=1, cols=70)
    assert r["z"].shape == r["n"].shape == r["h0"].shape == (40, 70) and not r["h0"].any()


def test_catchment_structure():
    """Tilted toward the south edge, Manning n from the four land-use classes,
    and a carved channel that never rises downstream."""
    from sw2d import scenarios as S
    s = S.catchment(256, dx=5.0, seed=2, amplitude=0.5)
    row_mean = s["z"].mean(axis=1)
    assert row_mean[0] > row_mean[-1] and np.corrcoef(np.arange(256), row_mean)[0, 1] < -0.95
    assert set(np.unique(s["n"])) <= set(S.MANNING_CLASSES)
    assert len(np.unique(s["n"])) == len(S.MANNING_CLASSES)
    # the channel: the lowest cell of every row, which descends row by row
    lowest = s["z"].min(axis=1)
    assert np.all(np.diff(lowest) <= 1e-12)
    scalar = S.catchment(64, seed=2, manning=0.04)
    assert scalar["n"] is None and scalar["manning"] == 0.04


def test_voronoi_fallback_matches_scipy(monkeypatch):
    """Without scipy (the numpy fallback) the roughness classes are the same."""
    from sw2d import scenarios as S
    pytest.importorskip("scipy")
    with_scipy = S._voronoi_classes(np.random.default_rng(7), 50, 61)
    real_import = builtins.__import__

    def no_scipy(name, *a, **k):
        if name.startswith("scipy"):
            raise ImportError(name)
        return real_import(name, *a, **k)

    monkeypatch.setattr(builtins, "__import__", no_scipy)
    without = S._voronoi_classes(np.random.default_rng(7), 50, 61)
    assert np.array_equal(with_scipy, without)


def test_ensemble_distribution():
    from sw2d import scenarios as S
    bank = S.TerrainBank(size=256, seed=3)
    e = S.ensemble(bank, count=40, sides=(32, 64, 128), seed=9, tail=1800.0)
    assert len(e) == 40 and {x["side"] for x in e} <= {32, 64, 128}
    for x in e:
        knots, kdt = x["rain"], x["rain_dt"]
        assert knots[0] == 0.0 and knots[2] == 0.0 and 20.0 <= knots[1] <= 120.0
        dur = 2.0 * kdt
        assert 900.0 <= dur <= 3600.0 and x["t_end"] == pytest.approx(dur + 1800.0)
        assert x["z"].shape == (x["side"], x["side"]) and x["n"].shape == x["z"].shape
    again = S.ensemble(bank, count=40, sides=(32, 64, 128), seed=9, tail=1800.0)
    assert all(np.array_equal(p["z"], q["z"]) for p, q in zip(e, again))


def test_request_stream_distribution():
    from sw2d import scenarios as S
    bank = S.TerrainBank(size=256, seed=3)
    r = S.request_stream(bank, rate=10.0, count=200, seed=4, side_min=32, side_max=256, horizon=(600.0, 900.0))
    arrivals = np.array([x["arrival"] for x in r])
    assert np.all(np.diff(arrivals) > 0)
    assert 0.07 < np.mean(np.diff(arrivals)) < 0.14  # mean inter-arrival 1/rate = 0.1 s
    sides = np.array([x["side"] for x in r])
    assert np.all(sides % 32 == 0) and sides.min() >= 32 and sides.max() <= 256
    assert len(np.unique(sides)) >= 4  # log-uniform over the range, not one size
    assert all(600.0 <= x["t_end"] <= 900.0 for x in r)
