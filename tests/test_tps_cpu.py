"""The treatment-planning environment's host side on the CPU: moqui's input-file rules
(mqi::file_parser), the tps_env keys and checks, and the output writers."""
import os

import numpy as np
import pytest

from moquimc_gb300 import tps

TEXT = """
## a tps input in moqui's format
GPUID 0
RandomSeed 1234   # fixed seed
randomseed 99     # a second line with the same key: the first one wins
Scorer Dose, LETd
SimulationType perBeam
ParticlesPerHistory 1000
RBE 1.1
NumberOfFraction 30
OutputDir {out}
OutputFormat mhd
OverwriteResults TRUE
StoppingStatistics 1
StoppingCriteria 1.5
StatThreshold 0.5
XShift 3.0
DensityScaling 1.035
BeamNumbers 2, 1
"""


def test_input_file_rules(tmp_path):
    p = tps.InputFile(TEXT.format(out=tmp_path))
    assert p.get_int("RandomSeed", -1) == 1234
    assert p.get_string("outputformat", "raw") == "mhd"        # keys are case-insensitive
    assert p.get_string("Missing", "dflt") == "dflt"
    assert p.get_bool("OverwriteResults", False) and p.get_bool("StoppingStatistics", False)
    assert not p.get_bool("Missing", False) and p.get_bool("Missing", True)
    assert p.get_string_vector("Scorer", ",") == ["Dose", "LETd"]
    assert p.get_float("XShift", 0.0) == 3.0 and p.get_float("YShift", 0.0) == 0.0
    assert p.get_int("NumberOfFraction", -1) == 30


def test_config_from_input(tmp_path):
    cfg = tps.TpsConfig.from_input(tps.InputFile(TEXT.format(out=tmp_path)))
    assert cfg.scorers == ["Dose", "LETd"] and cfg.simulation_type == "perBeam"
    assert cfg.random_seed == 1234 and cfg.n_fractions == 30 and cfg.output_format == "mhd"
    assert cfg.stopping_statistics and cfg.stopping_criteria == 1.5 and cfg.stat_threshold == 0.5
    # moqui's get_float returns a float: the values are FP32 roundings
    assert cfg.shift == (3.0, 0.0, 0.0) and cfg.density_scale == float(np.float32(1.035))
    assert cfg.beam_numbers == [2, 1]
    dij = tps.TpsConfig.from_input(tps.InputFile(f"Scorer Dij\nOutputDir {tmp_path}\n"))
    assert dij.simulation_type == "perSpot"                      # Dij forces per-spot runs
    for bad in (f"Scorer Dij, Dose\nOutputDir {tmp_path}\n", f"Scorer Heat\nOutputDir {tmp_path}\n",
                "Scorer Dose\n", f"OutputDir {tmp_path}\nStoppingStatistics true\n",
                f"OutputDir {tmp_path}\nStoppingStatistics true\nStoppingCriteria 1\n",
                f"OutputDir {tmp_path}\nCalibration custom\n"):
        with pytest.raises(ValueError):
            tps.TpsConfig.from_input(tps.InputFile(bad))


def test_output_writers(tmp_path):
    edges = (np.arange(5, dtype=np.float32) * 2.0 - 4.0, np.arange(4, dtype=np.float32) - 1.5,
             np.arange(3, dtype=np.float32) * 3.0)
    d = np.arange(4 * 3 * 2, dtype=np.float64)
    raw = tps.write_volume(str(tmp_path), "b_0_Dose", d, 2.5, "raw", edges)
    np.testing.assert_array_equal(np.fromfile(raw, np.float64), d * 2.5)
    mhd = tps.write_volume(str(tmp_path), "b_0_Dose", d, 2.5, "mhd", edges)
    head = open(mhd).read().splitlines()
    assert "TransformMatrix 1 0 0 0 1 0 0 0 1" in head and "Offset -3 -1 1.5" in head
    assert "DimSize = 4 3 2" in head and "ElementSpacing = 2 1 3" in head and "ElementDataFile = b_0_Dose.raw" in head
    np.testing.assert_array_equal(np.fromfile(os.path.join(tmp_path, "b_0_Dose.raw"), np.float64), d * 2.5)
    mha = tps.write_volume(str(tmp_path), "b_0_Dose", d, 2.5, "mha", edges)
    blob = open(mha, "rb").read()
    header_end = blob.index(b"ElementDataFile = LOCAL\n") + len(b"ElementDataFile = LOCAL\n")
    assert b"Origin = -3 -1 1.5\n" in blob[:header_end] and b"HeaderSize = -1\n" in blob[:header_end]
    np.testing.assert_array_equal(np.frombuffer(blob[header_end:], np.float64), d * 2.5)


def _write_mask(path, mask, dims):
    with open(path, "wb") as f:
        f.write(("ObjectType = Image\nNDims = 3\nDimSize = %d %d %d\nElementType = MET_UCHAR\n"
                 "ElementDataFile = LOCAL\n" % dims).encode())
        f.write(np.ascontiguousarray(mask, np.uint8).tobytes())


def test_mask_files_to_contour_roi(tmp_path):
    dims = (6, 4, 3)
    a = np.zeros(dims[::-1], np.uint8)
    b = np.zeros(dims[::-1], np.uint8)
    a[0, 1, 1:4] = 1          # one run of 3
    a[2, 3, 4:] = 1           # a run open at the end of the volume
    b[0, 1, 3:5] = 1          # overlaps a at one voxel (sum 2)
    pa, pb = os.path.join(tmp_path, "a.mha"), os.path.join(tmp_path, "b.mha")
    _write_mask(pa, a, dims)
    _write_mask(pb, b, dims)
    np.testing.assert_array_equal(tps.read_mask_mha(pa), a.reshape(-1))
    total = tps.read_mask_mha(pa).astype(np.uint16) + tps.read_mask_mha(pb)
    start, stride, acc = tps.mask_to_contour(total)
    # the summed mask along row (z=0, y=1) is 0 1 1 2 1 0: a run starts at x=1 and ends at x=5
    # (a voxel of sum 2 neither starts nor ends a run); the run at the end is closed there
    assert list(start) == [7, 70] and list(stride) == [4, 2] and list(acc) == [4, 6]
    np.testing.assert_array_equal(tps.contour_voxels(start, stride), [7, 8, 9, 10, 70, 71])
    with open(os.path.join(tmp_path, "bad.mha"), "w") as f:
        f.write("DimSize = 1 1 1\nElementDataFile = mask.raw\n")
    with pytest.raises(ValueError):
        tps.read_mask_mha(os.path.join(tmp_path, "bad.mha"))


def test_dij_npz_layout(tmp_path):
    """The Dij file in the reference's npz layout (save_to_npz / mqi::io::save_npz): members in
    its order with its dtypes, readable by scipy.sparse.load_npz as [n_spots, n_voxels]."""
    import zipfile

    from moquimc_gb300 import dij

    path = os.path.join(tmp_path, "b_1_Dij.npz")
    data = np.array([0.5, 1.5, 2.5, 4.0], np.float32)
    dij.write_dij_npz(path, np.array([0, 2, 2, 4], np.int64), np.array([1, 5, 0, 7]), data, 3, 8)
    with zipfile.ZipFile(path) as zf:
        assert [i.filename for i in zf.infolist()] == ["indices.npy", "indptr.npy", "shape.npy", "data.npy", "format.npy"]
        assert all(i.compress_type == zipfile.ZIP_STORED for i in zf.infolist())
    z = np.load(path)
    assert {k: z[k].dtype.str for k in z.files} == {"indices": "<u4", "indptr": "<u4", "shape": "<u4",
                                                   "data": "<f8", "format": "|S3"}
    assert z["format"].item() == b"csr" and list(z["shape"]) == [3, 8]
    sps = pytest.importorskip("scipy.sparse")
    m = sps.load_npz(path).toarray()
    want = np.zeros((3, 8))
    want[0, [1, 5]] = [0.5, 1.5]
    want[2, [0, 7]] = [2.5, 4.0]
    np.testing.assert_array_equal(m, want)
    with pytest.raises(ValueError):
        dij.write_dij_npz(path, np.array([0, 2]), np.array([1, 5, 0]), data[:3], 1, 8)
