"""The benchmark's reference arm on CPU: `bench.py --impl reference` times the
reference algorithm (the oracle's C restatement) on the host cores and prints
one JSON line with the keys the benchmark contract needs, without loading the
GPU library."""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


# runs bench.py's main, then reports whether the process mapped the GPU library
_RUNNER = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "config0", "--steps", "1",
            "--warmup", "0"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    assert not e.code, e.code
print("MAPPED_GPU_LIBRARY", "libfmf_gb300" in open("/proc/self/maps").read())
"""


@pytest.fixture(scope="module")
def run():
    if not os.path.exists("/proc/self/maps"):
        pytest.skip("needs /proc")
    p = subprocess.run([sys.executable, "-c", _RUNNER], capture_output=True, text=True, cwd=REPO,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return p.stdout


@pytest.fixture(scope="module")
def line(run):
    lines = [ln for ln in run.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, run[-2000:]
    return json.loads(lines[0])


def test_reference_arm_maps_no_gpu_library(run):
    assert "MAPPED_GPU_LIBRARY False" in run


def test_reference_line_has_the_contract_keys(line):
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"].startswith("config0")
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
    assert line["cpu_baseline"]["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
