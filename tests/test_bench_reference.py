"""The benchmark's reference arm on the CPU: `bench.py --impl reference` times the oracle (the
reference's BVESphereVelocity loop restated in C, src/SphereBVESolver.f90:395-420) on a bounded
block of the headline workload and prints one JSON line in the benchmark's format, with the
same metric and unit as the GPU arm, a cpu_baseline describing itself and an e2e with no
copies.  No GPU is involved."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def line(built_lib):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                          "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_reference_arm_line(line):
    assert line["impl"] == "reference"
    assert line["metric"].startswith("BVE direct-sum Ginteractions/s")
    assert line["unit"] == "Ginteractions/s" and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["steps"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["n_targets"] == 1966082 and line["config"]["n_sources"] == 1310720
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
