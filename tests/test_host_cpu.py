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


def test_npz_writer_of_the_host_drivers(tmp_path):
    """mqi_host::write_npz (the tps_env driver's Dij file): a stored zip of .npy members that numpy,
    zipfile's CRC check and scipy.sparse.load_npz read back, in the reference's member order and
    dtypes."""
    import zipfile

    src = tmp_path / "npz.cpp"
    src.write_text(r'''
#include "mqi_host.hpp"
int main(int, char** argv) {
    const uint32_t indices[4] = {1, 5, 0, 7}, indptr[4] = {0, 2, 2, 4}, shape[2] = {3, 8};
    const double   data[4] = {0.5, 1.5, 2.5, 4.0};
    mqi_host::write_npz(argv[1], {{"indices", "<u4", "(4,)", indices, sizeof(indices)},
                                  {"indptr", "<u4", "(4,)", indptr, sizeof(indptr)},
                                  {"shape", "<u4", "(2,)", shape, sizeof(shape)},
                                  {"data", "<f8", "(4,)", data, sizeof(data)},
                                  {"format", "|S3", "()", "csr", 3}});
    return 0;
}
''')
    exe = tmp_path / "npz"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT}/include", f"-I{ROOT}/moquimc_gb300/host", str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    path = tmp_path / "d.npz"
    subprocess.run([str(exe), str(path)], check=True)
    with zipfile.ZipFile(path) as zf:
        assert zf.testzip() is None
        assert [i.filename for i in zf.infolist()] == ["indices.npy", "indptr.npy", "shape.npy", "data.npy", "format.npy"]
    z = np.load(path)
    assert {k: z[k].dtype.str for k in z.files} == {"indices": "<u4", "indptr": "<u4", "shape": "<u4",
                                                   "data": "<f8", "format": "|S3"}
    sps = pytest.importorskip("scipy.sparse")
    m = sps.load_npz(str(path)).toarray()
    assert m.shape == (3, 8) and m[0, 1] == 0.5 and m[0, 5] == 1.5 and m[2, 0] == 2.5 and m[2, 7] == 4.0 and m.sum() == 8.5


def test_tps_driver_checks_its_input_before_touching_the_gpu(host_exe, tmp_path):
    """The C++ tps_env driver rejects the inputs tps_env rejects (Dij with other scorers, an unknown
    scorer, no OutputDir, StoppingStatistics without StoppingCriteria) with a message and status 1,
    before it creates a context."""
    exe = os.path.join(os.path.dirname(host_exe), "tps_env")
    cases = {"Scorer Dij, Dose\nOutputDir {o}\n": "Dij cannot be scored with the other quantities",
             "Scorer Heat\nOutputDir {o}\n": "Unrecognized scorer name",
             "Scorer Dose\n": "Output directory is not provided",
             "Scorer Dose\nOutputDir {o}\nStoppingStatistics true\n": "Statistical criteria must be positive"}
    for k, (text, msg) in enumerate(cases.items()):
        inp = tmp_path / f"in{k}.txt"
        inp.write_text(text.format(o=tmp_path / f"out{k}"))
        res = subprocess.run([exe, str(inp)], capture_output=True, text=True)
        assert res.returncode == 1 and msg in res.stderr, (text, res.stderr)
