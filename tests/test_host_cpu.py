"""The C++ host driver (moquimc_gb300/host/phantom_env_main.cpp): its beam source reproduces the
reference phantom_env's host-sampled vertices bit for bit (golden vectors from the reference's own
distribution classes), and its command line behaves like the reference's (required options)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def host_exe():
    from moquimc_gb300 import build

    build.build_all()
    exe = os.path.join(build.LIB_DIR, "phantom_env")
    assert os.path.exists(exe)
    return exe


def test_vertices_match_the_reference_beam_source(host_exe, tmp_path):
    g = np.load(os.path.join(GOLDEN, "vertices.npz"))
    hu = tmp_path / "ph.raw"
    np.zeros(8, np.int16).tofile(hu)
    k = 0
    while f"case{k}" in g:
        a = g[f"args{k}"]
        seed, gaus = int(a[0]), int(a[1])
        ref = g[f"case{k}"]
        out = tmp_path / f"v{k}.bin"
        cmd = [host_exe, "--nxyz", "2", "2", "2", "--phantom_path", str(hu), "--output_prefix", str(tmp_path),
               "--histories", str(len(ref)), "--random_seed", str(seed), "--beam", "gaussian" if gaus else "uniform",
               "--spot_position", *map(str, a[2:5]), "--spot_size", *map(str, a[5:7]), "--spot_energy", str(a[7]), "0",
               "--spot_angles", *map(str, a[8:12]), "--dump_vertices", str(out)]
        subprocess.run(cmd, check=True, capture_output=True)
        got = np.fromfile(out, np.float32).reshape(-1, 7)
        np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
        k += 1
    assert k >= 3


def test_required_options(host_exe, tmp_path):
    r = subprocess.run([host_exe, "--histories", "10"], capture_output=True, text=True)
    assert r.returncode != 0 and "output_path is required" in r.stderr
    r = subprocess.run([host_exe, "--output_prefix", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode != 0 and "phantom_path is required" in r.stderr
