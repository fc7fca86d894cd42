"""Autotuner: candidate search and the per-GPU cache (host logic on CPU, a
small real tuning run on the GPU)."""
import json

import pytest


def test_search_picks_fastest_and_skips_failures():
    from sw2d import autotune
    cands = [{"strip_h": s, "variant": v} for s in (16, 32, 64) for v in (0, 1)]

    def timer(c):
        if c["strip_h"] == 64 and c["variant"] == 1:
            raise RuntimeError("does not fit")
        return abs(c["strip_h"] - 32) + 0.1 * c["variant"] + 1.0

    best, table = autotune.search(cands, timer)
    assert best == {"strip_h": 32, "variant": 0}
    assert any("error" in r for r in table) and len(table) == len(cands)


def test_cache_roundtrip_and_size_classes(tmp_path):
    from sw2d import autotune
    p = tmp_path / "tune.json"
    c = autotune.Cache(str(p))
    cls = autotune.size_class(2048, 2048)
    assert cls == autotune.size_class(2000, 2100) and cls != autotune.size_class(1024, 1024)
    c.put("GB300", cls, {"strip_h": 48, "variant": 0})
    assert json.loads(p.read_text())["GB300"][cls]["strip_h"] == 48
    assert autotune.Cache(str(p)).get("GB300", cls) == {"strip_h": 48, "variant": 0}


@pytest.mark.gpu
def test_tune_small_grid_on_gpu(sw2d_mod, tmp_path):
    from sw2d import autotune
    cache = autotune.Cache(str(tmp_path / "t.json"))
    best = autotune.tune(256, 256, cache=cache, iters=12, strips=(16, 32), variants=(0, 4))
    assert best["strip_h"] in (16, 32) and best["variant"] in (0, 4)
    cfg = sw2d_mod.default_config(rows=256, cols=256, precision=sw2d_mod.PREC_F32, dt_mode=sw2d_mod.DT_CFL)
    autotune.apply(cfg, cache=cache)
    assert cfg.strip_h == best["strip_h"] and cfg.variant == best["variant"]
    g = sw2d_mod.Solver(cfg)  # the tuned configuration runs
    g.close()


def test_wave_strips_include_the_library_choice():
    """The autotuner's wave-fitting strips use the kernel's window width
    (27 output columns) and contain the strip the library picks itself:
    at 2048^2 on 152 SMs with the default 20-warp build, 76 column tiles x
    40 strips of 52 rows fill exactly one wave of 3040 warps (the
    decomposition sw2d_describe reports on GB300)."""
    from sw2d import autotune
    assert autotune.OUT_COLS == 27
    strips = autotune.wave_strips(2048, 2048, sms=152, waves=(1,), warps_per_sm=(20,))
    assert strips == [52]
    tiles = -(-2048 // autotune.OUT_COLS)
    assert tiles * -(-2048 // 52) == 152 * 20
    # more waves give shorter strips, never below 16 rows
    many = autotune.wave_strips(2048, 2048, sms=152)
    assert min(many) >= 16 and 52 in many and max(many) >= 52


@pytest.mark.gpu
def test_solver_takes_the_cached_choice(sw2d_mod, tmp_path, monkeypatch):
    """A cache entry for the size class changes the decomposition the library
    reports (sw2d_describe) for a handle created without an explicit one;
    an explicit strip height, or SW2D_AUTOTUNE=0, keeps the caller's."""
    from sw2d import autotune
    monkeypatch.setenv("SW2D_AUTOTUNE_CACHE", str(tmp_path / "t.json"))
    kw = dict(rows=256, cols=256, precision=sw2d_mod.PREC_F32, dt_mode=sw2d_mod.DT_CFL)
    with sw2d_mod.Solver(**kw) as g:
        before = g.describe()
    autotune.Cache().put(f"{autotune.gpu_name(0)}|{autotune.TABLE_VERSION}", autotune.size_class(256, 256),
                         {"strip_h": 24, "variant": 3})
    with sw2d_mod.Solver(**kw) as g:
        tuned = g.describe()
    assert "stream_step_kernel<8,2,1>" in tuned and "strip_h=24" in tuned and tuned != before
    with sw2d_mod.Solver(strip_h=32, **kw) as g:
        assert "strip_h=32" in g.describe()
    monkeypatch.setenv("SW2D_AUTOTUNE", "0")
    with sw2d_mod.Solver(**kw) as g:
        assert g.describe() == before


@pytest.mark.gpu
def test_batch_tuning_picks_a_build_and_chunk(sw2d_mod, tmp_path, monkeypatch):
    """tune_batch times builds of the batched kernel with graph chunks and a
    Batch created without them takes the choice; every build advances a
    scenario to the same bits (the arithmetic does not depend on the build)."""
    import numpy as np
    from sw2d import autotune
    from sw2d import scenarios as S
    monkeypatch.setenv("SW2D_AUTOTUNE_CACHE", str(tmp_path / "t.json"))
    best = autotune.tune_batch(variants=(0, 2), chunks=(6, 12), strips=(0, 64), count=4, launches=24)
    assert best["variant"] in (0, 2) and best["chunk"] in (6, 12) and best["strip_h"] in (0, 64)
    assert len(best["timings"]) == 5
    b = sw2d_mod.Batch(max_scenarios=4)
    assert (b.cfg.variant, b.cfg.chunk, b.cfg.strip_h) == (best["variant"], best["chunk"], best["strip_h"])
    b.close()
    s = S.catchment(96, dx=5.0, seed=2)
    depth = {}
    for v in (0, 1, 2):
        with sw2d_mod.Batch(variant=v, chunk=6, max_scenarios=2) as bt:
            cfg = sw2d_mod.default_config(rows=96, cols=96, dx=5.0, dy=5.0, precision=sw2d_mod.PREC_F32,
                                          dt_mode=sw2d_mod.DT_CFL, dt=1.0, south_open=1)
            sid = bt.add(cfg, s["z"], np.full((96, 96), 0.01), manning=s["n"], rain_kind=sw2d_mod.RAIN_STEP,
                         rain=np.array([60.0]), rain_dt=3600.0, t_end=120.0)
            while bt.advance(12):
                pass
            depth[v] = bt.field(sid)
    assert np.array_equal(depth[0], depth[1]) and np.array_equal(depth[0], depth[2])


def test_fixed_candidates_and_apply(tmp_path):
    """tune_fixed's candidates: every build at every iterations-per-launch
    with the library's strips, plus the one-launch choice of tune(); apply
    takes the fixed-step entry for a fixed-step config only, and leaves an
    explicit steps_per_launch alone."""
    import sw2d
    from sw2d import autotune
    c = autotune.fixed_candidates(1024, 1024, {"strip_h": 32, "variant": 2})
    assert {"strip_h": 0, "variant": 0, "steps_per_launch": 48} in c
    assert {"strip_h": 32, "variant": 2, "steps_per_launch": 1} in c
    assert len(c) == len(autotune.FIXED_VARIANTS) * len(autotune.STEPS_PER_LAUNCH) + 1
    cache = autotune.Cache(str(tmp_path / "t.json"))
    gpu = f"{autotune.gpu_name(0)}|{autotune.TABLE_VERSION}"
    cache.put(gpu, autotune.size_class(1024, 1024), {"strip_h": 32, "variant": 2})
    cache.put(gpu, autotune.fixed_class(1024, 1024), {"strip_h": 0, "variant": 0, "steps_per_launch": 96})
    cfl = sw2d.default_config(rows=1024, cols=1024, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_CFL)
    autotune.apply(cfl, cache=cache)
    assert (cfl.strip_h, cfl.variant, cfl.steps_per_launch) == (32, 2, 0)
    fx = sw2d.default_config(rows=1024, cols=1024, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_FIXED)
    autotune.apply(fx, cache=cache)
    assert (fx.strip_h, fx.variant, fx.steps_per_launch) == (0, 0, 96)
    fx1 = sw2d.default_config(rows=1024, cols=1024, precision=sw2d.PREC_F32, dt_mode=sw2d.DT_FIXED,
                              steps_per_launch=1)
    autotune.apply(fx1, cache=cache)
    assert fx1.steps_per_launch == 1


@pytest.mark.gpu
def test_tune_fixed_on_gpu(sw2d_mod, tmp_path):
    """A small real tuning run under the fixed time step picks one of its
    candidates, and a fixed-step Solver without a decomposition takes it."""
    from sw2d import autotune
    cache = autotune.Cache(str(tmp_path / "t.json"))
    best = autotune.tune_fixed(256, 256, cache=cache, iters=48, variants=(0,), steps=(1, 48))
    assert best["steps_per_launch"] in (1, 48) and best["variant"] == 0
    cfg = sw2d_mod.default_config(rows=256, cols=256, precision=sw2d_mod.PREC_F32, dt_mode=sw2d_mod.DT_FIXED, dt=0.1)
    autotune.apply(cfg, cache=cache)
    g = sw2d_mod.Solver(cfg)
    assert f"steps_per_launch={best['steps_per_launch']}" in g.describe()
    g.close()


def test_batch_tuning_then_strip_height_on_the_host(tmp_path, monkeypatch):
    """tune_batch picks the (build, chunk) pair with the size rule for the
    strips, then tries the taller strips for that pair only and keeps them
    when faster; apply_batch fills strip_h only where the caller left it to
    the library (fake timer, no GPU)."""
    from sw2d import autotune
    times = {(0, 12, 0): 3.0, (0, 24, 0): 2.0, (1, 12, 0): 2.5, (1, 24, 0): 2.2, (0, 24, 64): 1.9, (0, 24, 96): 1.7}
    seen = []

    def fake_timer(device, count, launches):
        def t(c):
            seen.append((c["variant"], c["chunk"], c["strip_h"]))
            return times[seen[-1]]
        return t

    monkeypatch.setattr(autotune, "_batch_timer", fake_timer)
    monkeypatch.setattr(autotune, "gpu_name", lambda device=0: "fake-gpu")
    monkeypatch.setenv("SW2D_AUTOTUNE_CACHE", str(tmp_path / "t.json"))
    best = autotune.tune_batch(variants=(0, 1), chunks=(12, 24), strips=(0, 64, 96))
    assert (best["variant"], best["chunk"], best["strip_h"]) == (0, 24, 96)
    assert seen[-2:] == [(0, 24, 64), (0, 24, 96)] and len(seen) == 6  # strips only for the best pair

    class B:  # the fields apply_batch reads and writes
        device, variant, chunk, strip_h = 0, 0, 0, 0

    b = autotune.apply_batch(B())
    assert (b.variant, b.chunk, b.strip_h) == (0, 24, 96)
    b = B()
    b.strip_h = 32
    assert autotune.apply_batch(b).strip_h == 32  # the caller's own strip height stays
    times[(0, 24, 64)] = times[(0, 24, 96)] = 9.0  # taller strips slower: the size rule stays
    best = autotune.tune_batch(variants=(0, 1), chunks=(12, 24), strips=(0, 64, 96), force=True)
    assert best["strip_h"] == 0
