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
