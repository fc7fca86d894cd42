"""bench.py's reference arm on the host cores: the JSON line's contract (keys,
units, steps, the zero-copy e2e of a CPU run) and the rank rule under
torchrun (rank 0 alone prints)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None, args=("--steps", "3", "--warmup", "3")):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_json_line():
    p = _run()
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "cell-updates/s" and d["unit"] == "cell-updates/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["grid"] == [2048, 2048]


def test_reference_arm_warmup_floor():
    """Fewer than 3 warm-up steps are raised to 3."""
    p = _run(args=("--steps", "1", "--warmup", "0"))
    assert p.returncode == 0, p.stderr[-2000:]
    d = json.loads([ln for ln in p.stdout.splitlines() if ln.startswith("{")][0])
    assert d["warmup"] == 3 and d["steps"] == 1


def test_reference_arm_other_ranks_print_nothing():
    p = _run({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert p.returncode == 0, p.stderr[-2000:]
    assert not [ln for ln in p.stdout.splitlines() if ln.startswith("{")]


def test_e2e_byte_counts_match_the_library_structs(tmp_path):
    """bench.py counts the e2e leg's copies with the sizes of the clock slot,
    the control block and the volume partials; they must be the library's."""
    import re
    import shutil
    import pytest
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    src = tmp_path / "sizes.cu"
    src.write_text('#include "sw2d_launch.h"\n#include <cstdio>\n'
                   'int main() { std::printf("%zu %zu %zu\\n", sizeof(sw2d::Clock), sizeof(sw2d::Control), '
                   '(size_t)sw2d::kVolumeBlocks * sizeof(double)); return 0; }\n')
    exe = tmp_path / "sizes"
    csrc = os.path.join(ROOT, "sw2d-gpu_gb300", "csrc")
    cc = subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", csrc, str(src), "-o",
                         str(exe)], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr[-2000:]
    clock_b, control_b, partials_b = map(int, subprocess.run([str(exe)], capture_output=True, text=True,
                                                              check=True).stdout.split())
    bench = open(os.path.join(ROOT, "bench.py")).read()
    m = re.search(r"clock_b, control_b, partials_b = (\d+), (\d+), (\d+) \* 8", bench)
    assert m, "bench.py's byte constants not found"
    assert (int(m.group(1)), int(m.group(2)), int(m.group(3)) * 8) == (clock_b, control_b, partials_b)


def test_depth_error_known_answers():
    """The accuracy figures bench.py reports (max |dh|, its 99.99th
    percentile, the flooded-area difference) on a constructed case."""
    import importlib.util
    import numpy as np
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    a = np.zeros((200, 50))
    a[:100] = 0.3                  # 5000 wet cells
    b = a.copy()
    b[5, :4] += 7e-4               # 4 cells differ by 0.7 mm
    b[150, 0] = 2e-4               # one cell wet in b only
    e = bench.depth_error(a, b)
    assert abs(e["max_abs_dh_m"] - 7e-4) < 1e-15
    assert e["flooded_area_rel_diff"] == 1 / 5000
    assert 0.0 <= e["p9999_abs_dh_m"] <= e["max_abs_dh_m"]
