"""Beamline children on the CPU: the host helpers (moquimc_gb300/beamline.py) against the
reference's own construction (tps_env::create_rangeshifter / create_voxelized_aperture, built by
oracle/ref_driver.cpp --beamline): aperture voxel densities and child rotations bit-exact."""
import json
import math
import os
import subprocess

import numpy as np
import pytest

from moquimc_gb300 import beamline as bl


def _run_reference(oracle, tmp_path, devices, histories=1):
    if not oracle.ref_available():
        pytest.skip("reference CPU build not available")
    path = os.path.join(tmp_path, "beamline.txt")
    oracle.write_beamline_file(path, devices)
    water = os.path.join(tmp_path, "water.raw")
    np.zeros((20, 20, 20), np.int16).tofile(water)
    cmd = oracle.ref_phantom_cmd(False, (20.0, 20.0, 20.0), (0.0, 0.0, -10.0), (20, 20, 20), 100.0, (0.0, 0.0, 100.0),
                                 (1.0, 1.0), histories, water, str(tmp_path), 1, "uniform", path)
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    with open(os.path.join(tmp_path, "run.json")) as f:
        return json.load(f)


def test_rotations_match_reference(oracle, tmp_path):
    angles = [(math.pi / 2, 0.0, 0.0), (0.3, 0.2, -1.1), (0.0, 2.0, 0.5), (0.0, 0.0, -0.7), (1.234, -0.5, 0.0)]
    devices = [("rangeshifter", (-5.0, -5.0, -1.0), (5.0, 5.0, 1.0), 1.19, a, (0.0, 0.0, 50.0 + 5 * k))
               for k, a in enumerate(angles)]
    rec = _run_reference(oracle, tmp_path, devices)
    for a, r in zip(angles, rec["beamline_rot"]):
        np.testing.assert_array_equal(bl.rotation_xyz(*a), np.array(r, np.float32))


def test_aperture_voxels_match_reference(oracle, tmp_path):
    square = np.array([[-20.0, -12.5], [20.0, -12.5], [20.0, 12.5], [-20.0, 12.5]], np.float32)
    devices = [
        ("aperture", (0.0, 0.0, 25.0), (120.0, 120.0, 10.0), [bl.circle(15.0)], (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)),
        # two openings: only the last one decides, as in the reference
        ("aperture", (3.0, -2.0, 40.0), (81.0, 60.5, 7.0), [bl.circle(10.0), square], (0.0, 0.0, 0.25),
         (1.0, 2.0, 3.0)),
    ]
    _run_reference(oracle, tmp_path, devices)
    mine = bl.children_from_devices(devices)
    for k, child in enumerate(mine):
        ref = np.fromfile(os.path.join(tmp_path, f"aperture{k}.bin"), np.float32)
        np.testing.assert_array_equal(child.rho, ref)
        assert (child.rho == bl.APERTURE_OPEN).any() and (child.rho == bl.APERTURE_BLOCK).any()
    # volume 81 x 60.5 x 7 at 1 mm: ceil per axis
    assert (len(mine[1].xe), len(mine[1].ye), len(mine[1].ze)) == (82, 62, 8)


def test_range_shifter_child():
    rs = bl.range_shifter((-100.0, -10.0, -100.0), (100.0, 10.0, 100.0), 1.19, bl.rotation_xyz(math.pi / 2, 0, 0),
                          (0.0, 0.0, 50.0))
    assert rs.rho.shape == (1,) and rs.rho[0] == np.float32(float(np.float32(1.19)) * 1e-3)
    np.testing.assert_array_equal(rs.ye, np.array([-10.0, 10.0], np.float32))
    # the rotation maps the child's y (20 mm) onto the world's z axis: a 20 mm slab across the beam
    r = rs.rot.reshape(3, 3)
    assert abs(abs(r[2, 1]) - 1.0) < 1e-6 and abs(r[2, 2]) < 1e-6
