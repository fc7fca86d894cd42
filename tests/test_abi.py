"""The C-ABI library on CPU: it builds, loads, exports every entry point
include/sw2d.h declares, and validates arguments before touching a GPU."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "sw2d.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sw2d_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_expected_entry_points():
    names = _declared()
    for n in ("sw2d_create", "sw2d_set_static", "sw2d_set_state", "sw2d_advance", "sw2d_get_field",
              "sw2d_get_budget", "sw2d_destroy"):
        assert n in names


def test_library_exports_every_declared_symbol(sw2d_mod):
    from sw2d import native
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (sw2d_[a-z0-9_]+)", out))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing
    # and the Python binding gives every one of them a signature
    assert sorted(native.exported_names()) == _declared()


def test_config_defaults_are_the_reference_constants(sw2d_mod):
    c = sw2d_mod.default_config()
    assert c.g == 9.80 and c.th == 1.0e-4 and c.precision == sw2d_mod.PREC_F64
    assert c.dt_mode == sw2d_mod.DT_FIXED and c.nodata == -9999.0


def test_invalid_configs_rejected_before_any_gpu_call(sw2d_mod):
    L = sw2d_mod.load()
    h = C.c_void_p()
    for kw in ({"rows": 0, "cols": 4}, {"rows": 4, "cols": 4, "dx": 0.0}, {"rows": 4, "cols": 4, "dt": -1.0},
               {"rows": 4, "cols": 4, "precision": 7}, {"rows": 4, "cols": 4, "dt_mode": 1, "cfl": 0.0},
               {"rows": 60000, "cols": 60000},  # beyond 32-bit field offsets
               {"rows": 2 ** 31 - 1, "cols": 4}, {"rows": 4, "cols": 2 ** 31 - 1}):  # int sums would overflow
        c = sw2d_mod.default_config(**kw)
        assert L.sw2d_create(C.byref(c), C.byref(h)) == 1
    assert L.sw2d_create(None, C.byref(h)) == 1


def test_batch_scenario_bytes_validates_its_arguments(sw2d_mod):
    """The admission estimate needs no GPU and refuses what sw2d_batch_add
    would refuse: a grid beyond 32-bit field offsets, a negative series."""
    L = sw2d_mod.load()
    n = C.c_int64()
    ok = sw2d_mod.default_config(rows=64, cols=64, precision=sw2d_mod.PREC_F32, dt_mode=sw2d_mod.DT_CFL)
    assert L.sw2d_batch_scenario_bytes(C.byref(ok), 3, 1, C.byref(n)) == 0 and n.value > 64 * 64 * 4
    for kw in ({"rows": 60000, "cols": 60000}, {"rows": 4, "cols": 2 ** 31 - 1}, {"rows": 0, "cols": 4}):
        c = sw2d_mod.default_config(**kw)
        assert L.sw2d_batch_scenario_bytes(C.byref(c), 3, 1, C.byref(n)) == 1
    assert L.sw2d_batch_scenario_bytes(C.byref(ok), -1, 1, C.byref(n)) == 1


def test_device_bytes(sw2d_mod):
    c64 = sw2d_mod.default_config(rows=2048, cols=2048)
    c32 = sw2d_mod.default_config(rows=2048, cols=2048, precision=sw2d_mod.PREC_F32)
    b64, b32 = sw2d_mod.device_bytes(c64), sw2d_mod.device_bytes(c32)
    assert b32 < b64
    assert b64 > 8 * 2049 * 2049 * 8


def test_status_strings(sw2d_mod):
    L = sw2d_mod.load()
    assert L.sw2d_status_string(0) == b"ok"
    assert L.sw2d_status_string(4) == b"non-finite value produced"


@pytest.mark.gpu
def test_describe_names_the_kernel_run(sw2d_mod):
    g = sw2d_mod.Solver(rows=300, cols=200, dx=1.0, dy=1.0)
    assert g.describe().startswith("step_kernel<double,")
    g.close()
    g = sw2d_mod.Solver(rows=300, cols=200, dx=1.0, dy=1.0, precision=sw2d_mod.PREC_F32, dt_mode=sw2d_mod.DT_CFL)
    d = g.describe()
    assert d.startswith("stream_step_kernel<") and "strip_h=" in d
    strip = int(d.split("strip_h=")[1].split()[0])
    units = int(d.split("units=")[1].split()[0])
    assert units == -(-200 // 27) * -(-300 // strip)  # column tiles x strips
    # the forcing build follows the forcing: uniform rain, then the storm build
    assert "forcing=uniform " in d
    g.set_storm(50.0, 0.0, 0.0, 1.0, 0.0, 100.0)
    assert "forcing=storm/sources " in g.describe()
    g.close()


C_CALLER = r"""
#include <math.h>
#include <stdio.h>
#include "sw2d.h"

int main(void) {
    sw2d_config cfg;
    if (sw2d_config_init(&cfg) != SW2D_OK) return 1;
    if (cfg.g != 9.80 || cfg.th != 1.0e-4 || cfg.precision != SW2D_PREC_F64) return 2;
    cfg.rows = 0; /* invalid: refused before any device call */
    sw2d_handle *h = NULL;
    if (sw2d_create(&cfg, &h) != SW2D_ERR_INVALID_ARG || h != NULL) return 3;
    int64_t n = 0;
    cfg.rows = cfg.cols = 64;
    cfg.dx = cfg.dy = 1.0;
    if (sw2d_device_bytes(&cfg, &n) != SW2D_OK || n <= 0) return 4;
    /* the serving loop's configuration, and a bad one refused before any device call */
    sw2d_server_config sc;
    if (sw2d_server_config_init(&sc) != SW2D_OK || sc.launches_per_step != 24 || sc.keep_depth != 1 ||
        sc.batch.max_scenarios < 1)
        return 5;
    sc.launches_per_step = 0;
    sw2d_server *srv = NULL;
    if (sw2d_server_create(&sc, &srv) != SW2D_ERR_INVALID_ARG || srv != NULL) return 6;
    int32_t state = -1;
    if (sw2d_server_poll(NULL, 1, &state, NULL, NULL) != SW2D_ERR_INVALID_ARG) return 7;
    printf("%s|%s|%lld\n", sw2d_status_string(SW2D_OK), sw2d_status_string(SW2D_ERR_NONFINITE), (long long)n);
    return 0;
}
"""


def test_header_compiles_as_c99_and_links(sw2d_mod, tmp_path):
    """A plain C99 caller (no C++ anywhere) includes the header, links the
    library and calls it: the extern "C" boundary as a C driver sees it."""
    from sw2d import native
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    lib_dir = os.path.dirname(native.LIB_PATH)
    cc = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I",
                         os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", lib_dir, "-lsw2d",
                         f"-Wl,-rpath,{lib_dir}", "-lm"], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, (run.returncode, run.stderr)
    ok, nonfinite, nbytes = run.stdout.strip().split("|")
    assert ok == "ok" and "non-finite" in nonfinite and int(nbytes) > 64 * 64 * 8


def test_invalid_batch_configs_rejected_before_any_gpu_call(sw2d_mod):
    from sw2d import native
    L = sw2d_mod.load()
    h = C.c_void_p()
    for kw in ({"chunk": 4}, {"chunk": 0}, {"max_scenarios": 0}, {"max_units": 0}, {"strip_h": -1}):
        c = native.batch_config(**kw)
        assert L.sw2d_batch_create(C.byref(c), C.byref(h)) == 1, kw
        assert not h.value
    assert L.sw2d_batch_create(None, C.byref(h)) == 1
    with pytest.raises(AttributeError):
        native.batch_config(no_such_field=1)
