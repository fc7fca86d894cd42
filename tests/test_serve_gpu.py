"""The serving loop on the GPU: requests arriving while others run are
admitted into the resident batch, and each result is bit-identical to the
same scenario run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone(sw2d_mod):
    from sw2d import scenarios as S
    from sw2d import serve
    bank = S.TerrainBank(size=256, seed=5)
    reqs_spec = S.request_stream(bank, rate=40.0, count=6, seed=7, side_min=32, side_max=160,
                                 horizon=(120.0, 400.0))

    def cfg(side):
        return sw2d_mod.default_config(rows=side, cols=side, dx=5.0, dy=5.0, precision=sw2d_mod.PREC_F32,
                                       dt_mode=sw2d_mod.DT_CFL, dt=2.0, cfl=0.5, south_open=1)

    reqs = [serve.Request(rid=k, arrival=s["arrival"], cfg=cfg(s["side"]), z=s["z"], depth=s["h0"], manning=s["n"],
                          rain_kind=sw2d_mod.RAIN_LINEAR, rain=s["rain"], rain_dt=s["rain_dt"], t_end=s["t_end"])
            for k, s in enumerate(reqs_spec)]
    bytes_of = lambda r: sw2d_mod.batch_scenario_bytes(r.cfg, 3, True)
    srv = serve.Server(lambda: sw2d_mod.Batch(chunk=6), bytes_of=bytes_of, max_bytes=int(1e9),
                       launches_per_tick=6, keep_results=True)
    st = srv.run(reqs, timeout=120.0)
    assert st["requests"] == len(reqs)
    assert st["p99_s"] >= st["p50_s"] > 0
    for r in srv.done:
        with sw2d_mod.Batch(chunk=6) as b:
            sid = b.add(r.cfg, r.z, r.depth, manning=r.manning, rain_kind=r.rain_kind, rain=r.rain,
                        rain_dt=r.rain_dt, t_end=r.t_end)
            while b.advance(12):
                pass
            alone = b.field(sid)
            assert b.poll()[sid]["steps"] == r.result["steps"]
        assert abs(r.result["t"] - r.t_end) < 1e-6
        assert np.array_equal(alone, r.result["depth"]), r.rid


def test_native_loop_served_results_equal_alone(sw2d_mod):
    """The same request stream through the library's own loop (NativeServer
    over sw2d_server_*): every result bit-identical to the scenario alone."""
    from sw2d import scenarios as S
    from sw2d import serve
    bank = S.TerrainBank(size=256, seed=5)
    reqs_spec = S.request_stream(bank, rate=40.0, count=6, seed=8, side_min=32, side_max=160,
                                 horizon=(120.0, 400.0))

    def cfg(side):
        return sw2d_mod.default_config(rows=side, cols=side, dx=5.0, dy=5.0, precision=sw2d_mod.PREC_F32,
                                       dt_mode=sw2d_mod.DT_CFL, dt=2.0, cfl=0.5, south_open=1)

    reqs = [serve.Request(rid=k, arrival=s["arrival"], cfg=cfg(s["side"]), z=s["z"], depth=s["h0"], manning=s["n"],
                          rain_kind=sw2d_mod.RAIN_LINEAR, rain=s["rain"], rain_dt=s["rain_dt"], t_end=s["t_end"])
            for k, s in enumerate(reqs_spec)]
    srv = serve.NativeServer(lambda: sw2d_mod.ServerHandle(chunk=6, launches_per_step=6, max_bytes=int(1e9)),
                             keep_results=True)
    st = srv.run(reqs, timeout=120.0)
    srv.close()
    assert st["requests"] == len(reqs) and st["failed"] == 0
    assert st["p99_s"] >= st["p50_s"] > 0 and 0 < st["peak_bytes"] <= int(1e9)
    for r in srv.done:
        with sw2d_mod.Batch(chunk=6) as b:
            sid = b.add(r.cfg, r.z, r.depth, manning=r.manning, rain_kind=r.rain_kind, rain=r.rain,
                        rain_dt=r.rain_dt, t_end=r.t_end)
            while b.advance(12):
                pass
            alone = b.field(sid)
            assert b.poll()[sid]["steps"] == r.result["steps"]
        assert abs(r.result["t"] - r.t_end) < 1e-6
        assert np.array_equal(alone, r.result["depth"]), r.rid
