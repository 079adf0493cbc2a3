"""The C++ host driver on the GPU: phantom_env_main run end to end writes the same dose as the
Python binding given the same vertices and seed, in the reference's file layout
(<output_prefix>/0_water_dE_total.raw, FP64, x fastest) and MetaImage headers."""
import os
import subprocess

import numpy as np
import pytest

from moquimc_gb300 import capi, phantom as ph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def host_exe(built_lib):
    from moquimc_gb300 import build

    build.build_all()
    return os.path.join(build.LIB_DIR, "phantom_env")


def test_host_driver_matches_the_binding(host_exe, tmp_path, gpu_ctx_factory):
    nxyz, lxyz, pxyz = (100, 100, 175), (100.0, 100.0, 350.0), (0.0, 0.0, -175.0)
    n, seed = 20000, 4321
    hu = np.zeros(nxyz[::-1], np.int16)
    hu[60:80] = 800                                     # a dense slab across the beam
    hp = tmp_path / "phantom.raw"
    hu.tofile(hp)
    args = [host_exe, "--lxyz", *map(str, lxyz), "--pxyz", *map(str, pxyz), "--nxyz", *map(str, nxyz),
            "--spot_position", "0", "0", "0.5", "--spot_size", "20", "20", "--spot_energy", "180", "0",
            "--histories", str(n), "--random_seed", str(seed), "--phantom_path", str(hp),
            "--output_prefix", str(tmp_path), "--output_format", "mhd", "--json", str(tmp_path / "run.json")]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert f"Number of particles tracked {n}" in r.stdout
    dose = np.fromfile(tmp_path / "0_water_dE_total.raw", np.float64)
    hdr = (tmp_path / "0_water_dE_total.mhd").read_text()
    assert "DimSize = 100 100 175" in hdr and "ElementType = MET_DOUBLE" in hdr
    subprocess.run(args + ["--dump_vertices", str(tmp_path / "v.bin")], check=True, capture_output=True)
    v = np.fromfile(tmp_path / "v.bin", np.float32).view(capi.VERTEX_DTYPE)
    c = gpu_ctx_factory()
    c.set_physics(True)
    cid = c.add_child(*ph.phantom_box_edges(lxyz, pxyz, nxyz))
    c.set_hu(cid, hu)
    sid = c.add_scorer(cid, capi.DOSE_W)
    c.set_vertices(v)
    c.transport(0, n, seed)
    np.testing.assert_allclose(dose, c.tally(sid), rtol=1e-12, atol=1e-300)
