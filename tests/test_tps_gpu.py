"""The treatment-planning environment on the GPU: a small CT, a synthetic beam model and two
beams run from an input file with moqui's keys; the written volumes against direct C-ABI runs of
the same plan and seed, statistical stopping, the Dij output and a beam-frame range shifter."""
import os

import numpy as np
import pytest

from moquimc_gb300 import capi, machine, phantom, tps

pytestmark = pytest.mark.gpu

MODEL = """
[geometry]
SAD(mm) 2000 1800
[spot]
90.0   90.2  0.7  5.0  5.2  0.003  0.003  1.0e5
130.0  130.3 0.7  4.2  4.4  0.0025 0.0025 1.0e5
170.0  170.1 0.6  3.6  3.7  0.002  0.002  1.0e5
"""


def _ct():
    nx, ny, nz = 60, 80, 40
    hu = np.zeros((nz, ny, nx), np.int16)
    hu[:, 30:36, :] = 900                      # a bone slab across the beam (along +y)
    edges = phantom.phantom_box_edges((120.0, 160.0, 80.0), (0.0, 0.0, 0.0), (nx, ny, nz))
    return hu, edges


def _beams(devices=()):
    spots = np.array([[e, x, z, 4.0] for e in (110.0, 140.0) for x in (-6.0, 0.0, 6.0) for z in (-6.0, 6.0)],
                     np.float32)
    return [tps.Beam("beam1", spots, devices=list(devices)), tps.Beam("Setup", spots[:1]),
            tps.Beam("beam2", spots[::2], gantry=10.0)]


def _env(tmp_path, extra, devices=()):
    text = f"RandomSeed 77\nScorer Dose, LETd\nParticlesPerHistory 1000\nNumberOfFraction 2\nOutputDir {tmp_path}\n"
    cfg = tps.TpsConfig.from_input(tps.InputFile(text + extra))
    hu, edges = _ct()
    return tps.TpsEnv(cfg, hu, edges, _beams(devices), machine.PBSMachine.parse(MODEL)), hu, edges


def test_tps_run_writes_scaled_volumes(tmp_path):
    env, hu, edges = _env(tmp_path, "OverwriteResults true\n")
    out = env.run()
    assert set(out) == {"beam1", "beam2"}                       # "Setup" is skipped
    n = int(np.prod(hu.shape))
    scale = 1000.0 * 1.1 * 2
    dose = np.fromfile(out["beam1"]["Dose"], np.float64)
    assert dose.size == n and dose.max() > 0
    for name in ("LETd_numer", "LETd_denom"):
        assert np.fromfile(out["beam1"][name], np.float64).size == n
    # the same plan, seed and scorers through the C ABI directly.  With three scorers on the CT
    # the reference's non-statistics kernel scores the first one (Dose) twice per step
    # (mqi_transport.hpp:204-225), and tps_env with "Scorer Dose, LETd" inherits that: so does
    # this environment, and a single dose scorer gives half the volume.
    m = machine.PBSMachine.parse(MODEL)
    plan = m.plan(env.beams[0].spots, -1.0, 390.0, (0.0, 0.0, 0.0, 90.0), (0.0, 0.0, 0.0), histories_from_ratio=1000.0)
    refs = {}
    for scorers in ((capi.DOSE_W, capi.LETD_NUM, capi.LETD_DEN), (capi.DOSE_W,)):
        c = capi.Context(0)
        try:
            c.set_physics(False)
            cid = c.add_child(*edges)
            c.set_hu(cid, hu)
            sid = [c.add_scorer(cid, t) for t in scorers][0]
            N = c.set_spot_plan(plan)
            c.transport_plan(0, N, 77)
            refs[len(scorers)] = c.tally(sid) * scale
        finally:
            c.close()
    np.testing.assert_allclose(dose, refs[3], rtol=1e-9, atol=1e-12 * refs[3].max())
    np.testing.assert_allclose(dose, 2.0 * refs[1], rtol=1e-9, atol=1e-12 * refs[1].max())
    # the beam travels along +y (iec2dicom) and stops in the CT: dose beyond the bone slab
    depth = dose.reshape(hu.shape).sum(axis=(0, 2))
    assert depth[:20].sum() > 0 and depth[40:].sum() > 0


def test_tps_statistical_stopping(tmp_path):
    env, _, _ = _env(tmp_path, "StoppingStatistics true\nStoppingCriteria 2.0\nStatThreshold 0.5\nBeamNumbers 1\n")
    out = env.run()
    assert list(out) == ["beam1"]
    assert int(out["beam1"]["passes"]) >= 1 and float(out["beam1"]["uncertainty"]) <= 0.02


def test_tps_dij_output(tmp_path):
    sps = pytest.importorskip("scipy.sparse")
    cfg = tps.TpsConfig.from_input(tps.InputFile(f"RandomSeed 5\nScorer Dij\nParticlesPerHistory 1000\n"
                                                 f"NumberOfFraction 1\nOutputDir {tmp_path}\nBeamNumbers 1\n"))
    hu, edges = _ct()
    out = tps.TpsEnv(cfg, hu, edges, _beams(), machine.PBSMachine.parse(MODEL)).run()
    z = np.load(out["beam1"]["Dij"])
    m = sps.csr_matrix((z["data"], z["indices"], z["indptr"]), shape=tuple(z["shape"]))
    assert m.shape[0] == 12 and m.nnz > 0


def test_tps_range_shifter_in_the_beam_frame(tmp_path):
    rs = [("rangeshifter", (-100.0, -100.0, 150.0), (100.0, 100.0, 180.0), 0.0, None, (0.0, 0.0, 0.0))]
    with_rs, hu, _ = _env(os.path.join(tmp_path, "a"), "RangeshifterDensity 1.19\nBeamNumbers 1\n", rs)
    without, _, _ = _env(os.path.join(tmp_path, "b"), "BeamNumbers 1\n")
    d1 = np.fromfile(with_rs.run()["beam1"]["Dose"], np.float64).reshape(hu.shape)
    d0 = np.fromfile(without.run()["beam1"]["Dose"], np.float64).reshape(hu.shape)
    assert os.path.exists(os.path.join(tmp_path, "a", "beam1_1_Dose.raw"))   # the CT is child 1
    # depth profiles from the entrance (the beam travels along +y)
    r1 = phantom.r80(d1.sum(axis=(0, 2)), 2.0)
    r0 = phantom.r80(d0.sum(axis=(0, 2)), 2.0)
    assert r0 - r1 > 20.0                                      # 30 mm of 1.19 g/cm^3 before the CT


def test_tps_scoring_mask(tmp_path):
    """ScoringMask with a mask file: the dose inside the mask equals the unmasked run's (same
    plan and seed), zero outside; the volume is written at the CT size."""
    hu, edges = _ct()
    mask = np.zeros(hu.shape, np.uint8)
    mask[10:30, 20:60, 20:40] = 1
    path = os.path.join(tmp_path, "target.mha")
    with open(path, "wb") as f:
        f.write(("ObjectType = Image\nNDims = 3\nDimSize = %d %d %d\nElementType = MET_UCHAR\n"
                 "ElementDataFile = LOCAL\n" % hu.shape[::-1]).encode())
        f.write(mask.tobytes())
    runs = {}
    for tag, extra in (("masked", f"ScoringMask true\nMask {path}\n"), ("full", "")):
        text = (f"RandomSeed 31\nScorer Dose\nParticlesPerHistory 1000\nNumberOfFraction 1\n"
                f"OutputDir {os.path.join(tmp_path, tag)}\nBeamNumbers 1\n" + extra)
        cfg = tps.TpsConfig.from_input(tps.InputFile(text))
        out = tps.TpsEnv(cfg, hu, edges, _beams(), machine.PBSMachine.parse(MODEL)).run()
        runs[tag] = np.fromfile(out["beam1"]["Dose"], np.float64).reshape(hu.shape)
    assert runs["masked"][mask == 0].max() == 0 and runs["masked"].max() > 0
    np.testing.assert_allclose(runs["masked"][mask == 1], runs["full"][mask == 1], rtol=1e-9,
                               atol=1e-12 * runs["full"].max())


def _write_beams(path, beams):
    """The C++ driver's beams file: beam lines, their spots and range shifters."""
    with open(path, "w") as f:
        for b in beams:
            f.write(f"beam {b.name} {b.gantry} {b.couch} {b.collimator} 0 0 0 390\n")
            for s in b.spots:
                f.write("spot " + " ".join(repr(float(v)) for v in s) + "\n")
            for d in b.devices:
                f.write("rangeshifter " + " ".join(repr(float(v)) for v in (*d[1], *d[2])) + "\n")


def _tps_exe():
    from moquimc_gb300 import build

    exe = os.path.join(build.LIB_DIR, "tps_env")
    if not os.path.exists(exe):
        build.build_host_tools()
    return exe


def test_cpp_tps_driver_matches_the_python_environment(tmp_path):
    """The C++ host driver (moquimc_gb300/host/tps_env_main.cpp) and the Python environment on the
    same input file, CT, beams and beam model write the same volumes."""
    import subprocess

    exe = _tps_exe()
    hu, edges = _ct()
    ct = os.path.join(tmp_path, "ct.raw")
    hu.tofile(ct)
    model = os.path.join(tmp_path, "model.txt")
    with open(model, "w") as f:
        f.write(MODEL)
    rs = ("rangeshifter", (-100.0, -100.0, 150.0), (100.0, 100.0, 180.0), 0.0, None, (0.0, 0.0, 0.0))
    beams = _beams([rs])
    _write_beams(os.path.join(tmp_path, "beams.txt"), beams)
    outs = {}
    for tag in ("cpp", "py"):
        text = (f"RandomSeed 42\nScorer Dose, LETt\nParticlesPerHistory 1000\nNumberOfFraction 3\nRBE 1.1\n"
                f"RangeshifterDensity 1.19\nDensityScaling 1.02\nXShift 1.5\nMachine PBS:{model}\n"
                f"OutputDir {os.path.join(tmp_path, tag)}\nOutputFormat mhd\n")
        inp = os.path.join(tmp_path, f"{tag}.in")
        with open(inp, "w") as f:
            f.write(text)
        if tag == "cpp":
            res = subprocess.run([exe, inp, "--ct", ct, "--ct_nxyz", "60", "80", "40", "--ct_lxyz", "120", "160", "80",
                                  "--ct_pxyz", "0", "0", "0", "--beams", os.path.join(tmp_path, "beams.txt")],
                                 capture_output=True, text=True)
            assert res.returncode == 0, res.stderr[-2000:]
        else:
            cfg = tps.TpsConfig.from_input(tps.InputFile.load(inp))
            tps.TpsEnv(cfg, hu, edges, beams, machine.PBSMachine.load(model)).run()
        outs[tag] = sorted(os.listdir(os.path.join(tmp_path, tag)))
    assert outs["cpp"] == outs["py"] and "beam1_1_Dose.raw" in outs["cpp"] and "beam2_0_LETt_numer.mhd" in outs["cpp"]
    for name in outs["cpp"]:
        a, b = (os.path.join(tmp_path, t, name) for t in ("cpp", "py"))
        if name.endswith(".raw"):
            x, y = np.fromfile(a, np.float64), np.fromfile(b, np.float64)
            np.testing.assert_allclose(x, y, rtol=1e-9, atol=1e-12 * max(np.abs(y).max(), 1e-30), err_msg=name)
        else:
            assert open(a).read() == open(b).read(), name


def test_cpp_tps_driver_dij_matches_the_python_environment(tmp_path):
    """Scorer Dij through the C++ driver and the Python environment on the same plan and seed: the
    same spot-row CSR in the reference's npz layout (the FP32 values to 1e-6: the FP64 table sums
    are accumulated in a different order)."""
    import subprocess

    exe = _tps_exe()
    hu, edges = _ct()
    ct = os.path.join(tmp_path, "ct.raw")
    hu.tofile(ct)
    model = os.path.join(tmp_path, "model.txt")
    with open(model, "w") as f:
        f.write(MODEL)
    beams = _beams()
    _write_beams(os.path.join(tmp_path, "beams.txt"), beams)
    got = {}
    for tag in ("cpp", "py"):
        text = (f"RandomSeed 9\nScorer Dij\nParticlesPerHistory 1000\nNumberOfFraction 1\nMachine PBS:{model}\n"
                f"OutputDir {os.path.join(tmp_path, tag)}\nBeamNumbers 1\n")
        inp = os.path.join(tmp_path, f"{tag}.in")
        with open(inp, "w") as f:
            f.write(text)
        if tag == "cpp":
            res = subprocess.run([exe, inp, "--ct", ct, "--ct_nxyz", "60", "80", "40", "--ct_lxyz", "120", "160", "80",
                                  "--ct_pxyz", "0", "0", "0", "--beams", os.path.join(tmp_path, "beams.txt")],
                                 capture_output=True, text=True)
            assert res.returncode == 0, res.stderr[-2000:]
        else:
            cfg = tps.TpsConfig.from_input(tps.InputFile.load(inp))
            tps.TpsEnv(cfg, hu, edges, beams, machine.PBSMachine.load(model)).run()
        got[tag] = np.load(os.path.join(tmp_path, tag, "beam1_0_Dij.npz"))
    a, b = got["cpp"], got["py"]
    assert sorted(a.files) == sorted(b.files)
    for k in ("indices", "indptr", "shape", "format"):
        assert a[k].dtype == b[k].dtype and np.array_equal(a[k], b[k]), k
    assert a["data"].dtype == np.float64 and a["data"].size > 0
    np.testing.assert_allclose(a["data"], b["data"], rtol=1e-6)
    assert list(a["shape"]) == [12, int(np.prod(hu.shape))]
