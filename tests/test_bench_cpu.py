"""bench.py's reference arm on the CPU: `--impl reference` runs the reference's own CPU build (one
process per host core) on the workload and prints one JSON line with the fields the measurement
contract names.  A tiny sample keeps it to seconds; the GPU arm is exercised by the GPU tests."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(oracle):
    if not oracle.ref_available():
        pytest.skip("the reference's staged sources are not present")
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c2",
                        "--steps", "1", "--warmup", "0", "--ref-histories", "20"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "primaries/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1
    assert d["config"]["workload"] == "c2_slab_phantom_150MeV"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "reference" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "primaries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
