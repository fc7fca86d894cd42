"""The reference's real-terrain dataset, peri_lake_model, end to end through
the reference-format driver (sw2d_run, FP64), against the CPU oracle run on
the same inputs read independently (tests/refio.py).

peri_lake_model (449 x 561 cells of 12.5 m, 122,307 of them active) has
NODATA borders, evaporation from temperature and radiation series, the
runoff fractions INT/INF/LWL with EV_WL_min, a -0.12 m^3/s sink, the
reference's rain formula and four WaterLevel probes.  Its setup.dat writes
an output every 3600 s (45,000 iterations); the copy used here writes one
every 30 s so that three outputs -- after the first iteration, at 30 s and
at 60 s -- take 750 iterations.  Everything else is the dataset as shipped.

Bar: every printed value of the three VTK files (depth, both velocities,
elevation, "%f") and of WaterLevel.txt equals the oracle's, character for
character.
"""
import os
import subprocess

import numpy as np
import pytest

import refio

GOLD = os.path.join(os.path.dirname(__file__), "golden", "peri_lake_db.tar.gz")
OUT_EVERY = 30.0  # s, output interval of the test copy of setup.dat


def _db(tmp_path):
    refio.extract(GOLD, tmp_path / "db")
    case = tmp_path / "db" / "peri_lake_model"
    (case / "output").mkdir()
    (tmp_path / "db" / "dir.txt").write_text("dir_number: 1\nperi_lake_model\n")
    setup = (case / "input" / "setup.dat").read_bytes().decode("latin-1").splitlines(keepends=True)
    out = []
    for line in setup:
        key = line.split(":", 1)[0].strip()
        out.append(f"{key}: {OUT_EVERY:g}\r\n" if key in ("dpout", "dkout") else line)
    (case / "input" / "setup.dat").write_bytes("".join(out).encode("latin-1"))
    return tmp_path / "db", case / "input"


def _oracle_inputs(O, inp):
    su = refio.read_setup(inp / "setup.dat")
    hdr, z = refio.read_esri(inp / "dem.txt")
    rows, cols = z.shape
    ic = np.array([float(x) for x in refio.tokens(inp / "initial_condition.txt")[: rows * cols]]).reshape(rows, cols)
    dtrain, rain, timmax = refio.read_rain(inp / "rain.dat")
    pts = refio.read_coords(inp / "coord_source_sink.dat")
    cells = np.array([refio.source_cell(hdr, rows, cols, x, y) for x, y in pts])
    q = refio.read_q(inp / "Q_source_sink.dat", len(pts))
    keep = (cells >= 0) & (cells < rows * cols)  # the reference writes past the grid into its padding row
    T, Rg, albedo = refio.read_evaporation_inputs(inp / "temperatures.txt", inp / "solar_radiation.txt")
    ev = O.evaporation_series(T, Rg, albedo, dtrain)
    o = O.Oracle(rows, cols, hdr["cellsize"], hdr["cellsize"], z, nodata=hdr["nodata_value"],
                 manning=su["manning_coef"][0], INT=su["INT"][0], INF=su["INF"][0], LWL=su["LWL"][0],
                 EV_WL_min=su["EV_WL_min"][0], dt_mode=0, dt=su["dt"][0])
    o.set_state(ic)
    o.set_forcing(O.OracleForcing(rain_kind=O.RAIN_COMPAT, rain=rain, rain_dt=dtrain, ev=ev, ev_dt=dtrain,
                                  sources=cells[keep], src_q=q[:, keep], dtoq=su["dtoq"][0]))
    probes = sorted(refio.probe_cell(hdr, rows, cols, x, y) for x, y in refio.read_coords(inp / "coord_out.dat"))
    return o, hdr, z, ic, timmax, su, probes


def test_peri_lake_inputs_as_the_reference_reads_them():
    """The dataset's shape and forcing, as the test reads them (no GPU)."""
    import tempfile
    from pathlib import Path
    with tempfile.TemporaryDirectory() as d:
        _, inp = _db(Path(d))
        hdr, z = refio.read_esri(inp / "dem.txt")
        assert z.shape == (561, 449) and hdr["cellsize"] == 12.5
        assert int(np.sum(z != hdr["nodata_value"])) == 122307
        dtrain, rain, timmax = refio.read_rain(inp / "rain.dat")
        assert dtrain == 3600.0 and rain.size == 817 and timmax == 816 * 3600.0
        su = refio.read_setup(inp / "setup.dat")
        assert su["evaporation_on"][0] == 1 and su["dpout"][0] == OUT_EVERY and su["dt"][0] == 0.04
        pts = refio.read_coords(inp / "coord_source_sink.dat")
        assert len(pts) == 1 and np.all(refio.read_q(inp / "Q_source_sink.dat", 1) == -0.12)
        assert len(refio.read_coords(inp / "coord_out.dat")) == 4


@pytest.mark.gpu
def test_peri_lake_driver_matches_oracle(sw2d_mod, oracle_mod, tmp_path):
    import build_native
    db, inp = _db(tmp_path)
    r = subprocess.run([build_native.DRIVER, "--db", str(db), "--precision", "f64", "--max-outputs", "3"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = db / "peri_lake_model" / "output"
    o, hdr, z, ic, timmax, su, probes = _oracle_inputs(oracle_mod, inp)
    rows, cols = z.shape
    fmt = np.vectorize(lambda v: "%f" % v, otypes=[object])
    per_out = int(round(OUT_EVERY / su["dt"][0])) // 2  # iterations between outputs (two half steps each)
    wl = (out / "WaterLevel.txt").read_text().split("\n")
    done = 0
    for k, iters in enumerate((1, per_out - 1, per_out)):
        assert o.advance(iters, timmax) == iters
        done += iters
        h = ic if k == 0 else o.state()["h"]  # the first VTK prints the initial depth (cu:1415-1420)
        uu, vv = o.cell_velocity()
        got = refio.read_vtk_fields(out / f"Results_{k}.vtk", rows, cols)
        assert np.array_equal(got["depth"], fmt(h)), k
        assert np.array_equal(got["x_velocity"], fmt(vv)), k
        assert np.array_equal(got["y_velocity"], fmt(-uu)), k
        assert np.array_equal(got["Elevations"], fmt(z)), k
        assert wl[k] == "".join(" %f" % h.ravel()[c] for c in probes), k
    assert done == 2 * per_out
    assert not (out / "Results_3.vtk").exists()
    # the run moved water: evaporation, sink and rain all acted on the lake
    assert not np.array_equal(o.state()["h"], ic)
