"""The reference-format host driver (sw2d_run) end to end.

The reference's own dam_break case (inputs and its shipped Results_0.vtk,
tests/golden/dam_break_db.tar.gz) runs through the driver; the VTK the
driver writes must equal the reference's byte for byte."""
import os
import subprocess
import tarfile

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "dam_break_db.tar.gz")


def _db(tmp_path):
    with tarfile.open(GOLD) as tf:
        tf.extractall(tmp_path / "db")
    os.rename(tmp_path / "db" / "dam_break" / "output" / "Results_0.vtk", tmp_path / "reference_Results_0.vtk")
    (tmp_path / "db" / "dir.txt").write_text("dir_number: 1\ndam_break\n")
    return tmp_path / "db"


def _driver(sw2d_mod):
    import build_native
    return build_native.DRIVER


def test_driver_rejects_bad_arguments(sw2d_mod):
    r = subprocess.run([_driver(sw2d_mod), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
def test_driver_reproduces_reference_vtk_byte_for_byte(sw2d_mod, tmp_path):
    db = _db(tmp_path)
    r = subprocess.run([_driver(sw2d_mod), "--db", str(db), "--max-outputs", "1"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = (db / "dam_break" / "output" / "Results_0.vtk").read_bytes()
    ref = (tmp_path / "reference_Results_0.vtk").read_bytes()
    assert got == ref
    assert (db / "dam_break" / "output" / "WaterLevel.txt").read_text() == "Outlet off\n"
    assert (db / "dam_break" / "output" / "TimeSimu_0.txt").exists()


@pytest.mark.gpu
def test_driver_second_output_matches_oracle(sw2d_mod, oracle_mod, tmp_path):
    """The output at 60 s (mstep = lkout) against the oracle run on the
    same inputs, compared at the VTK's printed precision."""
    db = _db(tmp_path)
    r = subprocess.run([_driver(sw2d_mod), "--db", str(db), "--max-outputs", "2"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = db / "dam_break" / "output" / "Results_1.vtk"
    assert out.exists() and not (db / "dam_break" / "output" / "Results_2.vtk").exists()
    txt = out.read_text().split("\n")
    k = txt.index("SCALARS depth float 1") + 2
    depth = np.array([float(x) for x in txt[k:k + 10000]]).reshape(100, 100)[::-1]
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "dam_break.npz"))
    o = oracle_mod.Oracle(100, 100, 10.0, 10.0, d["z"], manning=float(d["manning"]), INT=float(d["INT"]),
                          INF=float(d["INF"]), LWL=float(d["LWL"]), EV_WL_min=float(d["EV_WL_min"]), dt_mode=0,
                          dt=0.04)
    o.set_state(d["h0"])
    assert o.advance(750, 6000.0) == 750
    ref = np.array([float("%f" % v) for v in o.state()["h"].ravel()]).reshape(100, 100)
    assert np.array_equal(depth, ref)


@pytest.mark.gpu
def test_driver_roughness_raster_and_outflow_hydrograph(sw2d_mod, oracle_mod, tmp_path):
    """Extensions: input/manning.txt (per-cell n) and --south-open with the
    outflow hydrograph file; the 60 s depth and outflow volume against the
    oracle run with the same raster and open edge."""
    db = _db(tmp_path)
    case = db / "dam_break"
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "dam_break.npz"))
    n = 0.010 + 0.040 * np.repeat(np.arange(100)[:, None] / 99.0, 100, axis=1)
    head = (case / "input" / "dem.txt").read_text().split("\n")[:6]
    body = "\n".join(" ".join("%.6f" % v for v in row) for row in n)
    (case / "input" / "manning.txt").write_text("\n".join(head) + "\n" + body + "\n")
    n = np.array([[float("%.6f" % v) for v in row] for row in n])
    r = subprocess.run([_driver(sw2d_mod), "--db", str(db), "--south-open", "--max-outputs", "3"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    txt = (case / "output" / "Results_1.vtk").read_text().split("\n")
    k = txt.index("SCALARS depth float 1") + 2
    depth = np.array([float(x) for x in txt[k:k + 10000]]).reshape(100, 100)[::-1]
    o = oracle_mod.Oracle(100, 100, 10.0, 10.0, d["z"], n=n, manning=float(d["manning"]), INT=float(d["INT"]),
                          INF=float(d["INF"]), LWL=float(d["LWL"]), EV_WL_min=float(d["EV_WL_min"]), dt_mode=0,
                          dt=0.04, south_open=1)
    o.set_state(d["h0"])
    assert o.advance(750, 6000.0) == 750
    ref = np.array([float("%f" % v) for v in o.state()["h"].ravel()]).reshape(100, 100)
    assert np.array_equal(depth, ref)
    lines = (case / "output" / "Outflow.txt").read_text().strip().split("\n")
    assert lines[0].split() == ["time_s", "outflow_volume_m3", "outflow_rate_m3_per_s"]
    rows = [[float(x) for x in l.split()] for l in lines[1:]]
    assert len(rows) == 3
    assert all(b[1] >= a[1] for a, b in zip(rows, rows[1:]))  # cumulative volume never decreases
    assert rows[1][1] == pytest.approx(o.budget()["outflow"], rel=1e-9, abs=1e-9)



@pytest.mark.gpu
def test_driver_rain_weights_raster(sw2d_mod, oracle_mod, tmp_path):
    """Extension: input/rain_weights.txt distributes rain.dat's rain over the
    cells; the 60 s depth against the oracle with the same factors and the
    reference's rain formula."""
    db = _db(tmp_path)
    case = db / "dam_break"
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "dam_break.npz"))
    rain = [6.0, 12.0, 3.0, 0.0, 9.0] + [0.0] * 60
    lines = ["60.0\t", "Time (min)\tRainfall (mm)"] + ["%d\t%g" % (k + 1, v) for k, v in enumerate(rain)]
    (case / "input" / "rain.dat").write_text("\r\n".join(lines) + "\r\n")
    w = np.array([[float("%.4f" % v) for v in row] for row in
                  np.random.default_rng(4).uniform(0.0, 4.0, (100, 100))])
    head = (case / "input" / "dem.txt").read_text().split("\n")[:6]
    body = "\n".join(" ".join("%.4f" % v for v in row) for row in w)
    (case / "input" / "rain_weights.txt").write_text("\n".join(head) + "\n" + body + "\n")
    r = subprocess.run([_driver(sw2d_mod), "--db", str(db), "--max-outputs", "2"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    txt = (case / "output" / "Results_1.vtk").read_text().split("\n")
    k = txt.index("SCALARS depth float 1") + 2
    depth = np.array([float(x) for x in txt[k:k + 10000]]).reshape(100, 100)[::-1]
    o = oracle_mod.Oracle(100, 100, 10.0, 10.0, d["z"], manning=float(d["manning"]), INT=float(d["INT"]),
                          INF=float(d["INF"]), LWL=float(d["LWL"]), EV_WL_min=float(d["EV_WL_min"]), dt_mode=0,
                          dt=0.04)
    o.set_state(d["h0"])
    o.set_forcing(oracle_mod.OracleForcing(rain_kind=oracle_mod.RAIN_COMPAT, rain=np.array(rain), rain_dt=60.0,
                                           rain_w=w))
    assert o.advance(750, 6000.0) == 750
    ref = np.array([float("%f" % v) for v in o.state()["h"].ravel()]).reshape(100, 100)
    assert np.array_equal(depth, ref)
    # against uniform rain the depth changed
    o2 = oracle_mod.Oracle(100, 100, 10.0, 10.0, d["z"], manning=float(d["manning"]), INT=float(d["INT"]),
                           INF=float(d["INF"]), LWL=float(d["LWL"]), EV_WL_min=float(d["EV_WL_min"]), dt_mode=0,
                           dt=0.04)
    o2.set_state(d["h0"])
    o2.set_forcing(oracle_mod.OracleForcing(rain_kind=oracle_mod.RAIN_COMPAT, rain=np.array(rain), rain_dt=60.0))
    o2.advance(750, 6000.0)
    assert not np.array_equal(o2.state()["h"], o.state()["h"])
