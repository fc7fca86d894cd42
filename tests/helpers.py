"""Shared drivers for the parity tests: the same seeded scenario through the
CPU oracle and through the C ABI of libsw2d.so."""
import numpy as np


def make_pair(O, sw2d, rows, cols, dx, z, h0, n=None, manning=0.0, precision=0, dt_mode=1, dt=1.0,
              cfl=0.5, south_open=0, nodata=-9999.0, INT=0.0, INF=0.0, LWL=0.0, EV_WL_min=0.0, dy=None,
              tile=None):
    dy = dx if dy is None else dy
    o = O.Oracle(rows, cols, dx, dy, z, n=n, nodata=nodata, manning=manning, INT=INT, INF=INF, LWL=LWL,
                 EV_WL_min=EV_WL_min, dt_mode=dt_mode, dt=dt, cfl=cfl, south_open=south_open)
    o.set_state(h0)
    kw = {}
    if tile:
        kw = {"tile_h": tile[0], "tile_w": tile[1]}
    g = sw2d.Solver(rows=rows, cols=cols, dx=dx, dy=dy, nodata=nodata, manning=manning, INT=INT, INF=INF,
                    LWL=LWL, EV_WL_min=EV_WL_min, precision=precision, dt_mode=dt_mode, dt=dt, cfl=cfl,
                    south_open=south_open, **kw)
    g.set_static(z, n)
    g.set_state(h0)
    return o, g


def set_forcing(O, o, g, rain_kind=0, rain=None, rain_dt=1.0, storm=None, ev=None, ev_dt=1.0,
                sources=None, src_q=None, dtoq=1.0):
    kind = O.RAIN_STORM if storm is not None else rain_kind
    o.set_forcing(O.OracleForcing(rain_kind=kind, rain=rain, rain_dt=rain_dt, storm=storm, ev=ev,
                                  ev_dt=ev_dt, sources=sources, src_q=src_q, dtoq=dtoq))
    if storm is not None:
        g.set_storm(storm["peak"], storm["x0"], storm["y0"], storm["vx"], storm["vy"], storm["sigma"],
                    storm.get("tstop", 1e300))
    elif rain_kind:
        g.set_rain(rain_kind, rain, rain_dt)
    if ev is not None:
        g.set_evaporation(ev, ev_dt)
    if sources is not None:
        g.set_point_sources(sources, src_q, dtoq)


def compare(o, g):
    a = o.state()
    b = g.state()
    return a, b


def same(x, y):
    """Equal values (+0 and -0 count as equal), NaN nowhere."""
    return bool(np.array_equal(x, y))


def max_abs(x, y):
    return float(np.max(np.abs(x - y))) if x.size else 0.0
