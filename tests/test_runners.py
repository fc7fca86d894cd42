"""The command-line runners the ncu summaries were made with run on small
cases and print their throughput line."""
import os
import re
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sw2d-gpu_gb300", "sw2d")


def _run(script, *args):
    r = subprocess.run([sys.executable, os.path.join(PKG, script), *args], capture_output=True, text=True,
                       timeout=600, env=dict(os.environ, SW2D_AUTOTUNE="0"))
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_runcase_prints_throughput():
    out = _run("runcase.py", "--precision", "f32", "--size", "128", "--iters", "4")
    assert re.search(r"iters=4 .* cell-updates/s \(host timed\); stream_step_kernel<", out), out


def test_runbatch_prints_throughput():
    out = _run("runbatch.py", "--count", "4", "--iters", "8", "--sides", "64", "128")
    m = re.search(r"scenarios=4 iters=8 launches=(\d+) .* ([0-9.e+]+) cell-updates/s \(host timed\)", out)
    assert m, out
    assert int(m.group(1)) == 56 and float(m.group(2)) > 0  # 48 warm-up iterations, then 8
