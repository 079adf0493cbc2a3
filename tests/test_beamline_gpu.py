"""Beamline children on the GPU against the reference's CPU build: a 20 mm range shifter (a
single-voxel child rotated 90 degrees about x, so that its 20 mm axis lies along the beam) and a
voxelised aperture with a 15 mm-radius opening, in front of a water phantom; a 150 MeV beam with a
uniform +-30 mm profile.  The reference puts the same children before its phantom
(oracle/ref_driver.cpp --beamline, built as tps_env builds them).  Depth dose and lateral profile
within 2% or 3 sigma in bins above 10% of the maximum (>= 95% of bins), R80 within 0.3 mm; the
shifter pulls R80 in by more than 15 mm and the aperture stops most of the beam."""
import math
import os

import numpy as np
import pytest

from moquimc_gb300 import beamline as bl
from moquimc_gb300 import capi
from moquimc_gb300 import phantom as ph

pytestmark = pytest.mark.gpu

LXYZ, PXYZ, NXYZ = (100.0, 100.0, 200.0), (0.0, 0.0, -100.0), (100, 100, 200)
ENERGY, SPOT_POS, SPOT_SIZE = 150.0, (0.0, 0.0, 100.0), (30.0, 30.0)
DEVICES = [
    ("rangeshifter", (-100.0, -10.0, -100.0), (100.0, 10.0, 100.0), 1.19, (math.pi / 2, 0.0, 0.0), (0.0, 0.0, 50.0)),
    ("aperture", (0.0, 0.0, 25.0), (120.0, 120.0, 10.0), [bl.circle(15.0)], (0.0, 0.0, 0.0), (0.0, 0.0, 0.0)),
]
BATCHES, EACH = 8, 4000


def _lateral(d):
    nx, ny, nz = NXYZ
    return d.reshape(nz, ny, nx).sum(axis=0).reshape(ny // 5, 5, nx // 5, 5).sum(axis=(1, 3))


def _agree(a, b):
    am, as_ = a.mean(0), a.std(0, ddof=1) / np.sqrt(len(a))
    bm, bs = b.mean(0), b.std(0, ddof=1) / np.sqrt(len(b))
    sel = bm > 0.1 * bm.max()
    ok = (np.abs(am - bm) <= 0.02 * bm) | (np.abs(am - bm) <= 3 * np.sqrt(as_ ** 2 + bs ** 2))
    return ok[sel].mean()


def _gpu(make, devices, seed0):
    c = make()
    c.set_physics(False)
    for child in bl.children_from_devices(devices):
        child.add_to(c)
    cid = c.add_child(*ph.phantom_box_edges(LXYZ, PXYZ, NXYZ))
    c.set_hu(cid, np.zeros(NXYZ[::-1], np.int16))
    sid = c.add_scorer(cid, capi.DOSE_W)
    idd, lat = [], []
    for b in range(BATCHES):
        v = ph.uniform_spot_vertices(EACH, np.random.default_rng(seed0 + b), ENERGY, SPOT_POS, SPOT_SIZE)
        c.reset()
        c.set_vertices(v)
        c.transport(0, EACH, seed0 * 31 + b)
        d = c.tally(sid)
        idd.append(ph.depth_dose(d, NXYZ) / EACH)
        lat.append(_lateral(d) / EACH)
    return np.array(idd), np.array(lat)


def test_beamline_children_match_reference(oracle, gpu_ctx_factory, tmp_path):
    if not oracle.ref_available():
        pytest.skip("reference CPU build not available")
    path = os.path.join(tmp_path, "beamline.txt")
    oracle.write_beamline_file(path, DEVICES)
    _, _, doses = oracle.ref_phantom_parallel(False, LXYZ, PXYZ, NXYZ, ENERGY, SPOT_POS, SPOT_SIZE, EACH, BATCHES,
                                              np.zeros(NXYZ[::-1], np.int16), 600, "uniform",
                                              workdir=str(tmp_path), beamline=path)
    r_idd = np.array([ph.depth_dose(d, NXYZ) / EACH for d in doses])
    r_lat = np.array([_lateral(d) / EACH for d in doses])
    g_idd, g_lat = _gpu(gpu_ctx_factory, DEVICES, 700)
    assert _agree(g_idd, r_idd) >= 0.95
    assert _agree(g_lat, r_lat) >= 0.95
    r80_ref, r80_gpu = ph.r80(r_idd.mean(0), 1.0), ph.r80(g_idd.mean(0), 1.0)
    assert abs(r80_gpu - r80_ref) <= 0.3, (r80_gpu, r80_ref)
    # physical sanity: without the shifter the range is longer; without the aperture far more dose
    o_idd, o_lat = _gpu(gpu_ctx_factory, DEVICES[1:], 800)
    assert ph.r80(o_idd.mean(0), 1.0) - r80_gpu > 15.0
    n_idd, _ = _gpu(gpu_ctx_factory, DEVICES[:1], 900)
    assert n_idd.mean(0).sum() > 3.0 * g_idd.mean(0).sum()
