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
  * the largest offset fits the kernel's 32-bit element offsets;
  * for the pipelined launches (sw2d_pipe.cuh), every domain cell a unit
    reads or writes is owned by a unit at most one column tile and one strip
    away, once strips have kPipeMinStrip rows: the neighbour set each unit
    waits for covers all it depends on.
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
    assert "ld_state(Hin + gp - 1)" in unit and "ld_state(Hin + gp + 1)" in unit
    assert "ld_state(Rin + gp - 3 * pitch)" in unit
    assert "r_first = R0 - 4, r_last = R1 + 3" in unit
    return dict(top=top, bottom=bottom, left=left, pitch=lambda c: ((c + pa + pb) // 32) * 32, hl=hl, hr=hr)


def _strips_even(rows, strip_h):
    """The single-scenario kernels' split (strip_rows in sw2d_stream.cuh):
    ceil(rows / strip_h) strips whose heights differ by at most one row."""
    n = -(-rows // strip_h)
    q, rem = divmod(rows, n)
    out, r0 = [], 0
    for rs in range(n):
        r1 = r0 + q + (1 if rs < rem else 0)
        out.append((r0, r1))
        r0 = r1
    return out


def _strip_start(rows, n, skew, k):
    """strip_start of sw2d_stream.cuh in Python integers."""
    return (rows * k * 200 * n + skew * rows * k * (n - k) + 100 * n * n) // (200 * n * n)


def _strips_skew(rows, strip_h, skew=20):
    """The single-scenario kernel's skewed split: ceil(rows / strip_h)
    strips whose heights fall by `skew` percent from the first to the last."""
    n = -(-rows // strip_h)
    b = [_strip_start(rows, n, skew, k) for k in range(n + 1)]
    return list(zip(b[:-1], b[1:]))


def _strips_fixed(rows, strip_h):
    """The batched kernel's split: strips of strip_h rows, the last shorter."""
    return [(r0, min(r0 + strip_h, rows)) for r0 in range(0, rows, strip_h)]


def _check(rows, cols, strip_h, K, split=_strips_even):
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
        for r0, r1 in split(rows, strip_h):
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
    K = _consts()
    _check(rows, cols, strip_h, K, _strips_even)
    _check(rows, cols, strip_h, K, _strips_fixed)


def test_skewed_split_matches_the_kernel_source_and_covers_the_rows():
    """The model's skewed split is the kernel's formula; it starts at row 0,
    ends at `rows`, has no empty strip and falls monotonically, for the
    shapes the library skews (one full wave, mean height >= 16)."""
    src = open(os.path.join(CSRC, "sw2d_stream.cuh")).read()
    assert "return (int)((R * kk * 200 * n + skew * R * kk * (n - kk) + 100 * n * n) / (200 * n * n));" in src
    api = open(os.path.join(CSRC, "sw2d_api.cu")).read()
    skew = int(re.search(r"constexpr int kStripSkew = (\d+);", api).group(1))
    K = _consts()
    for rows, sh in ((2048, 52), (2048, 16), (4096, 103), (1000, 17), (16, 16), (33, 16), (8192, 137)):
        sp = _strips_skew(rows, sh, skew)
        assert sp[0][0] == 0 and sp[-1][1] == rows
        assert all(a[1] == b[0] for a, b in zip(sp, sp[1:]))
        hs = [r1 - r0 for r0, r1 in sp]
        assert min(hs) >= 1 and all(x >= y - 1 for x, y in zip(hs, hs[1:]))  # falling, up to rounding
        assert max(hs) <= round(sh * (1 + skew / 200)) + 1
        _check(rows, 2049, sh, K, lambda r, s_: _strips_skew(r, s_, skew))


def test_even_split_matches_the_kernel_source():
    """The model's split is the one strip_rows writes."""
    src = open(os.path.join(CSRC, "sw2d_stream.cuh")).read()
    assert "r0 = rs * q + min(rs, rem);" in src and "r1 = r0 + q + (rs < rem ? 1 : 0);" in src
    for rows, sh in ((2048, 52), (17, 16), (9, 16), (150, 16), (101, 10)):
        sp = _strips_even(rows, sh)
        assert sp[0][0] == 0 and sp[-1][1] == rows and len(sp) == -(-rows // sh)
        assert all(a[1] == b[0] for a, b in zip(sp, sp[1:]))
        assert max(r1 - r0 for r0, r1 in sp) <= sh and max(r1 - r0 for r0, r1 in sp) - min(r1 - r0 for r0, r1 in sp) <= 1


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


def _pipe_min_strip():
    pipe = open(os.path.join(CSRC, "sw2d_pipe.cuh")).read()
    return int(re.search(r"constexpr int kPipeMinStrip = (\d+);", pipe).group(1))


def _check_pipe_neighbours(rows, cols, strip_h, K):
    """Owners (column tile, strip) of every domain cell that unit (ct, rs)
    reads -- rows R0-7 .. R1+2 (the remainder of row r-3 is read with row r),
    columns gj0-1 .. gj0+32 -- or writes: all within one tile and one strip."""
    out = 32 - K["hl"] - K["hr"]
    tiles_w = -(-cols // out)
    sp = _strips_even(rows, strip_h)
    owner = np.concatenate([np.full(r1 - r0, k) for k, (r0, r1) in enumerate(sp)])  # strip of each row
    for ct in range(tiles_w):
        gj0 = ct * out - K["hl"]
        c_lo, c_hi = max(gj0 - 1, 0), min(gj0 + 32, cols - 1)
        t_lo, t_hi = c_lo // out, c_hi // out
        assert ct - 1 <= t_lo and t_hi <= ct + 1, (rows, cols, ct)
        for rs, (r0, r1) in enumerate(sp):
            rr_lo, rr_hi = max(r0 - 7, 0), min(r1 + 2, rows - 1)
            s_lo, s_hi = owner[rr_lo], owner[rr_hi]
            assert rs - 1 <= s_lo and s_hi <= rs + 1, (rows, cols, strip_h, rs)


@pytest.mark.parametrize("cols", [1, 27, 28, 55, 200, 2049])
@pytest.mark.parametrize("rows", [8, 9, 40, 150, 2048])
def test_pipe_neighbour_set_covers_the_window(rows, cols):
    """Every strip height whose even split keeps strips of at least
    kPipeMinStrip rows (the condition the library checks)."""
    K = _consts()
    m = _pipe_min_strip()
    for strip_h in sorted({m, m + 1, 12, 16, 52, rows}):
        n = -(-rows // strip_h)
        if n == 1 or rows // n >= m:
            _check_pipe_neighbours(rows, cols, strip_h, K)


def test_pipe_neighbour_model_needs_the_minimum_strip():
    """Strips of 6 rows let a unit read a strip two away, which no wait
    covers: the model must see that."""
    K = _consts()
    m = _pipe_min_strip()
    with pytest.raises(AssertionError):
        _check_pipe_neighbours(64, 60, m - 2, K)
    with pytest.raises(AssertionError):  # 60 rows in 10 strips of 6
        _check_pipe_neighbours(60, 60, 6, K)
