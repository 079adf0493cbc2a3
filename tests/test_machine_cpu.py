"""The pencil-beam machine model (moquimc_gb300/machine.py) on the CPU.

moqui's pbs class cannot be built here (its headers include the DICOM library), so the beam-model
parsing and interpolation are checked against the formulas of mqi_treatment_machine_pbs.hpp
written out in FP32, and the beam's coordinate_transform against the reference's own beam source
(oracle/ref_driver.cpp vertices: the same draws with and without the angles)."""
import math
import os
import subprocess

import numpy as np
import pytest

from moquimc_gb300 import capi
from moquimc_gb300 import machine as mm

f = np.float32

MODEL = """
# a synthetic beam model in moqui's generic PBS format
[geometry]
SAD(mm) 2000 1800          # x, y
rangeshifter(mm) 300 0
aperture(mm) 0 0
[rangeshifter_thickness]
"RS_40" 40.0
[spot]
# nominal  E      dE    x    y    xp     yp     ratio
70.0      70.2   0.8   6.0  6.5  0.003  0.0035 1.0e5
100.0     100.3  0.7   4.5  4.8  0.0025 0.003  1.2e5
150.0     150.1  0.6   3.5  3.6  0.002  0.0024 1.5e5
[time]
I(nA) 2.0
E(sec) 1.5
"""


def _intpl(x, x0, x1, y0, y1):
    x, x0, x1, y0, y1 = (f(v) for v in (x, x0, x1, y0, y1))
    return y0 if x1 == x0 else f(y0 + (x - x0) * (y1 - y0) / (x1 - x0))


def test_parse_beam_model():
    m = mm.PBSMachine.parse(MODEL)
    assert m.sad == (2000.0, 1800.0)
    assert list(m.beamdata) == [70.0, 100.0, 150.0]
    assert m.beamdata[100.0].E == float(f(100.3)) and m.beamdata[150.0].ratio == float(f(1.5e5))
    assert m.rangeshifter_thickness == {"RS_40": 40.0}
    assert m.time["I(nA)"] == 2.0 and m.rangeshifter == (300.0, 0.0)
    par = mm.PBSMachine.parse(MODEL.replace("SAD(mm) 2000 1800", "SAD(mm) 0 0"))
    assert par.sad == (math.inf, math.inf)


def test_interpolation_matches_the_reference_formulas():
    m = mm.PBSMachine.parse(MODEL)
    e = 123.4
    p = m.spot_parameters(e)
    d, u = m.beamdata[100.0], m.beamdata[150.0]
    assert p["E"] == _intpl(e, 100.0, 150.0, d.E, u.E)
    assert p["ratio"] == _intpl(e, 100.0, 150.0, d.ratio, u.ratio)
    for k in ("dE", "x", "y", "xp", "yp"):   # against the rows' E, as characterize_beamlet does
        assert p[k] == _intpl(e, d.E, u.E, getattr(d, k), getattr(u, k)), k
    assert m.histories(e, 3.0, 100.0) == int(f(f(3.0) * f(p["ratio"]) / f(100.0)))
    for bad in (70.0, 60.0, 150.5):
        with pytest.raises(ValueError):
            m.spot_parameters(bad)


def test_beam_start_points_back_to_the_virtual_source():
    m = mm.PBSMachine.parse(MODEL)
    beam, d = m.beam_start(40.0, -30.0, 390.0)
    assert beam[2] == f(390.0)
    assert beam[0] == f(f(40.0) * (f(2000.0) - f(390.0)) / f(2000.0))
    assert beam[1] == f(f(-30.0) * (f(1800.0) - f(390.0)) / f(1800.0))
    assert abs(float(np.linalg.norm(d)) - 1.0) < 1e-6 and d[2] < 0
    # the ray from the start through the isocentre point comes from the virtual source (0, 0, SAD)
    t = (2000.0 - 390.0) / -d[2]
    assert abs(beam[0] - t * d[0]) < 1e-3
    par = mm.PBSMachine.parse(MODEL.replace("SAD(mm) 2000 1800", "SAD(mm) 0 0"))
    b2, d2 = par.beam_start(40.0, -30.0, 390.0)
    assert b2[0] == f(40.0) and b2[1] == f(-30.0) and np.allclose(d2, [0, 0, -1])


def test_plan_fields_and_histories():
    m = mm.PBSMachine.parse(MODEL)
    spots = [(80.0, 10.0, 5.0, 0.2), (140.0, -20.0, 0.0, 1.3)]
    plan = m.plan(spots, particles_per_history=1000.0, angles=(0.0, 90.0, 0.0, 0.0), isocenter=(1.0, 2.0, 3.0))
    assert plan.dtype == capi.SPOT_DTYPE and len(plan) == 2
    assert list(plan["histories"]) == [math.ceil(float(f(0.2)) * 1000.0), math.ceil(float(f(1.3)) * 1000.0)]
    p = m.spot_parameters(140.0)
    assert plan[1]["energy"] == p["E"] and plan[1]["energy_sigma"] == p["dE"]
    assert list(plan[1]["sigma"]) == [p["x"], p["y"], 0.0, p["xp"], p["yp"]]
    assert list(plan[1]["trans"]) == [1.0, 2.0, 3.0]
    assert list(m.plan(spots, particles_per_history=-1)["histories"]) == [1, 1]
    by_ratio = m.plan(spots, histories_from_ratio=50.0)
    assert by_ratio[0]["histories"] == m.histories(80.0, 0.2, 50.0)


def test_coordinate_rotation_matches_reference_beam_source(oracle, tmp_path):
    """The reference's beam source with angles = coordinate_transform(angles).rotation applied to
    the same draws without angles (pos' = R pos, dir' = R dir, mqi_beamlet.hpp:80-90), bit for bit."""
    if not oracle.ref_available():
        pytest.skip("reference CPU build not available")

    def draw(angles):
        out = os.path.join(tmp_path, "v.bin")
        cmd = [oracle.ref_binary(False), "vertices", out, "64", "5", "1", "3.0", "-2.0", "390.0", "4.0", "5.0",
               "120.0", *map(str, angles)]
        subprocess.run(cmd, check=True, capture_output=True)
        return oracle.read_vecs(out, [np.float32])[0].reshape(-1, 7)

    base = draw((0.0, 0.0, 0.0, 0.0))
    for angles in ((0.0, 90.0, 0.0, 0.0), (15.0, 45.0, -30.0, 90.0), (0.0, 270.0, 10.0, -90.0)):
        rot = mm.coordinate_rotation(angles).reshape(3, 3)
        got = draw(angles)
        for cols in ((1, 2, 3), (4, 5, 6)):
            v = base[:, cols]
            r = (rot[:, 0] * v[:, :1] + rot[:, 1] * v[:, 1:2]) + rot[:, 2] * v[:, 2:3]
            np.testing.assert_array_equal(r.astype(np.float32), got[:, cols], err_msg=str(angles))
