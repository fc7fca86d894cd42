"""FP64 parity on the benchmark configurations themselves, at their stated
sizes, through the C ABI against the CPU oracle.

C1 (the plain method at small size): the 1D-in-2D dam break on a flat,
frictionless 256 x 512 channel (x along the 512 columns), dx = dy = 1 m,
10 m of water for x < 256 m and dry downstream, reflective walls, no rain,
2000 iterations under the CFL-0.5 rule.

C2 crop: a 512 x 512 window of the seeded 2048 x 2048 catchment (the bench's
terrain: tilted fractal DEM with the carved channel, Manning n per cell from
the Voronoi land-use classes) at its south edge, which is open, with the
channel crossing it; dry at the start, 50 mm/h of rain, 300 iterations (every
cell crosses the wet/dry threshold on the way).
Friction makes every face evaluate the power h^(4/3): the FP64 path uses the
oracle's own deterministic log/exp, so the bar stays bit for bit.

Bar: bit-identical depth and discharges, same time and iteration count.
"""
import numpy as np
import pytest

from helpers import make_pair, max_abs, same, set_forcing

pytestmark = pytest.mark.gpu

TH = 1.0e-4


def _check_bitwise(o, g):
    a, b = o.state(), g.state()
    assert same(a["h"], b["h"]), max_abs(a["h"], b["h"])
    assert same(a["um"], b["um"]), max_abs(a["um"], b["um"])
    assert same(a["vn"], b["vn"]), max_abs(a["vn"], b["vn"])
    bud = g.budget()
    assert bud["t"] == a["t"] and bud["steps"] == a["steps"]
    return a


def test_c1_dam_break_512x256_2000_iterations_bitwise(oracle_mod, sw2d_mod):
    from sw2d import scenarios as S
    s = S.dam_break_channel(256, 512, 1.0, h_up=10.0, x_gate=256.0)
    o, g = make_pair(oracle_mod, sw2d_mod, 256, 512, 1.0, s["z"], s["h0"], dt_mode=1, dt=1.0, cfl=0.5)
    assert abs(2.0 * o.next_dt() - 0.5 / np.sqrt(98.0)) < 1e-12  # the first step: CFL 0.5 over sqrt(g * 10 m)
    assert o.advance(2000) == 2000
    assert g.advance(2000) == 2000
    a = _check_bitwise(o, g)
    # the bore and the rarefaction have travelled: the front is well past the gate; with walls all round
    # the volume changes only by what the depth clamp at the front added
    front = int(np.max(np.nonzero(a["h"][128] > 1e-3)[0]))
    assert 300 < front < 512
    gain = o.budget()["clamp_gain"]
    assert abs((a["h"].sum() - s["h0"].sum()) - gain) <= 1e-9 * s["h0"].sum()
    assert g.budget()["clamp_gain"] == pytest.approx(gain, rel=1e-6)


@pytest.fixture(scope="module")
def c2_crop():
    from sw2d import scenarios as S
    full = S.catchment(2048, dx=5.0, seed=20240)
    r0, c0 = 2048 - 512, 1280  # the channel runs through columns 1407..1632 of the last 512 rows
    z = full["z"][r0:, c0:c0 + 512].copy()
    n = full["n"][r0:, c0:c0 + 512].copy()
    bare = S.catchment(2048, dx=5.0, seed=20240, channel=False)["z"][r0:, c0:c0 + 512]
    assert np.all(np.any(z != bare, axis=1))  # the carved channel crosses every row of the window
    return z, n


def test_c2_catchment_crop_512_bitwise(oracle_mod, sw2d_mod, c2_crop):
    z, n = c2_crop
    assert len(np.unique(n)) == 4  # all four land-use classes in the window
    h0 = np.zeros(z.shape)  # the configuration starts dry
    o, g = make_pair(oracle_mod, sw2d_mod, 512, 512, 5.0, z, h0, n=n, south_open=1, dt_mode=1, dt=1.0, cfl=0.5)
    set_forcing(oracle_mod, o, g, rain_kind=2, rain=np.array([50.0, 50.0]), rain_dt=3600.0)
    assert o.advance(300) == 300
    assert g.advance(300) == 300
    a = _check_bitwise(o, g)
    # every cell is wet by now and water leaves through the open south edge
    assert np.all(a["h"] > TH)
    bo, bg = o.budget(), g.budget()
    assert bo["outflow"] > 0.0
    assert bg["outflow"] == pytest.approx(bo["outflow"], rel=1e-9)
