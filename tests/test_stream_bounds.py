"""The FP32 streaming kernel reads without bounds tests, relying on the zero
frame around every field.  This checks that reasoning on the host, for many
grid shapes, with the constants taken from the sources themselves
(sw2d_launch.h: frame and pitch; sw2d_stream_unit.cuh: halo lanes):

  * every column is an output of exactly one (column tile, lane);
  * every element a warp reads -- rows R0-4 .. R1+2, the window's columns
    and the neighbour columns loaded at its edges, the remainder of row
    r-3 -- lies inside its allocation and inside its own row;
  * every element it writes (the output rows and the south-face copy) lies
    inside the allocation;
  * the largest offset fits the kernel's 32-bit element offsets.
"""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sw2d-gpu_gb300", "csrc")


def _consts():
    launch = open(os.path.join(CSRC, "sw2d_launch.h")).read()
    unit = open(os.path.join(CSRC, "sw2d_stream_unit.cuh")).read()
    top, bottom, left = map(int, re.search(
        r"kGhostTop = (\d+), kGhostBottom = (\d+), kGhostLeft = (\d+);", launch).groups())
    pa, pb = map(int, re.search(r"pitch_for\(int cols\) \{ return \(\(cols \+ (\d+) \+ (\d+)\) / 32\) \* 32;",
                                launch).groups())
    hl = int(re.search(r"constexpr int kStreamHL = (\d+);", unit).group(1))
    hr = int(re.search(r"constexpr int kStreamHR = (\d+);", unit).group(1))
    # the loads: the window's column, one to the west and one to the east
    assert "Hin[gp - 1]" in unit and "Hin[gp + 1]" in unit and "Rin[gp - 3 * pitch]" in unit
    assert "r_first = R0 - 4, r_last = R1 + 3" in unit
    return dict(top=top, bottom=bottom, left=left, pitch=lambda c: ((c + pa + pb) // 32) * 32, hl=hl, hr=hr)


def _check(rows, cols, strip_h, K):
    pitch = K["pitch"](cols)
    out = 32 - K["hl"] - K["hr"]
    origin = K["top"] * pitch + K["left"]
    plane = (K["top"] + rows + 1 + K["bottom"]) * pitch
    lo, hi = -origin, plane - origin  # valid element offsets relative to cell (0,0)
    tiles_w = -(-cols // out)
    lanes = np.arange(32)
    owner = np.zeros(cols, dtype=int)
    max_off = 0
    for ct in range(tiles_w):
        gj0 = ct * out - K["hl"]
        gj = gj0 + lanes
        is_out = (lanes >= K["hl"]) & (lanes < K["hl"] + out) & (gj < cols)
        np.add.at(owner, gj[is_out], 1)
        # columns read on any row: gj - 1 .. gj + 1, all inside the row's span
        cmin, cmax = int(gj.min()) - 1, int(gj.max()) + 1
        assert cmin >= -K["left"], (rows, cols, ct, cmin)
        assert cmax <= pitch - K["left"] - 1, (rows, cols, ct, cmax, pitch)
        for rs in range(-(-rows // strip_h)):
            r0 = rs * strip_h
            r1 = min(r0 + strip_h, rows)
            rmin, rmax = r0 - 4, r1 + 2  # rows loaded
            assert rmin >= -K["top"] and rmax <= rows + K["bottom"]
            first, last = rmin * pitch + cmin, rmax * pitch + cmax
            assert lo <= first and last < hi
            # the remainder of row lrow-3 is read only when lrow >= 3
            assert max(rmin, 3) - 3 >= 0
            # writes: output rows r0 .. r1-1 and, for the last row, the copy below it
            wlast = (r1 if r1 == rows else r1 - 1) * pitch + min(int(gj[is_out].max(initial=0)), cols - 1)
            assert wlast < hi
            max_off = max(max_off, last + origin, wlast + origin)
    assert np.all(owner == 1), (rows, cols)
    assert max_off < 2 ** 31


@pytest.mark.parametrize("cols", [1, 2, 26, 27, 28, 31, 32, 53, 54, 55, 64, 65, 96, 97, 127, 128, 129, 200, 2048,
                                  2049, 8192])
@pytest.mark.parametrize("rows, strip_h", [(1, 16), (5, 16), (40, 16), (64, 52), (150, 16), (2048, 52)])
def test_stream_windows_cover_once_and_stay_in_the_frame(rows, cols, strip_h):
    _check(rows, cols, strip_h, _consts())


@pytest.mark.parametrize("cols", [28, 55, 2053])
def test_the_bounds_model_catches_a_narrow_frame(cols):
    """The last window reaches furthest when it holds a single output column
    (cols = 1 modulo the output width): its east neighbour load is then
    29 columns past the east wall, so a row needs cols + 33 elements with
    the 4-column west frame.  One element fewer must fail the model, so the
    check above is not vacuous."""
    K = _consts()
    out = 32 - K["hl"] - K["hr"]
    assert cols % out == 1
    _check(8, cols, 16, K)
    K["pitch"] = lambda c: c + 32
    with pytest.raises(AssertionError):
        _check(8, cols, 16, K)
