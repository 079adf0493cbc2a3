"""The moqui-side binding on the GPU: moqui's phantom example run through phantom_env_gb300 (moqui's
own phantom_env class, host beam source and save_reshaped_files, with run()/finalize() on the C
ABI) writes the same 0_water_dE_total.raw as this repository's C++ host driver on the same command
line: the vertices are the reference's in both, the transport the same kernels and random streams,
so the doses agree to FP64 summation order.  (moqui's phantom_env always writes raw; the host
driver's --output_format is its own addition, and the writers are compared byte for byte on the
CPU.)"""
import os
import subprocess

import numpy as np
import pytest

from test_binding_cpu import REF_SRC, build_binding

pytestmark = pytest.mark.gpu

ARGS = ["--lxyz", "100", "100", "350", "--pxyz", "0", "0", "-175", "--nxyz", "100", "100", "175", "--spot_energy",
        "200", "0", "--spot_position", "0", "0", "0.5", "--spot_size", "30", "30", "--histories", "20000",
        "--random_seed", "7"]


def test_binding_matches_the_host_driver(tmp_path):
    if not os.path.isdir(os.path.join(REF_SRC, "moqui")):
        pytest.skip("the reference's staged sources are not present")
    from moquimc_gb300 import build

    build.build_all()
    exe = build_binding(str(tmp_path), True)
    ph = tmp_path / "water.raw"
    np.zeros((175, 100, 100), np.int16).tofile(ph)
    outs = {}
    for name, prog in (("binding", exe), ("host", os.path.join(build.LIB_DIR, "phantom_env"))):
        d = tmp_path / name
        d.mkdir()
        r = subprocess.run([prog, *ARGS, "--phantom_path", str(ph), "--output_prefix", str(d)],
                           capture_output=True, text=True)
        assert r.returncode == 0, (name, r.stderr[-2000:])
        outs[name] = d
    a = np.fromfile(outs["binding"] / "0_water_dE_total.raw", np.float64)
    b = np.fromfile(outs["host"] / "0_water_dE_total.raw", np.float64)
    assert a.size == b.size == 100 * 100 * 175 and a.sum() > 0
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-300)
