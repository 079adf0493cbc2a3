"""The Dij npz against the reference's own code, on the CPU.

* The reference's table (insert_hashtable's CPU branch, moqui/kernel_functions/mqi_transport.hpp:
  68-111) and writer (save_to_npz, moqui/base/mqi_io.hpp:249-320, over mqi::io::save_npz,
  moqui/base/mqi_sparse_io.hpp:167-399), fed with a list of insertions, give one entry per distinct
  (voxel, spot) key with a positive value, and nothing for values <= 0.
* The C++ host writer (mqi_host::write_npz, the tps_env driver's Dij file) writes the same bytes as
  the reference's writer for the four numeric members (local header, .npy header, payload, central
  directory record).  The string member "format" holds "csr" in both; the reference writes it as
  sizeof(std::string) bytes per character read from the string's buffer (96 bytes, 93 of them
  whatever memory follows), so only its header and first three bytes are compared.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        pytest.skip("the reference's staged sources are not present")
    return oracle


def _insertions(seed=3, n=20000, n_spots=7, n_vox=5000):
    rng = np.random.default_rng(seed)
    vox = rng.integers(0, n_vox, n).astype(np.uint32)
    spot = rng.integers(0, n_spots, n).astype(np.uint32)
    val = rng.exponential(1e-3, n)
    val[rng.random(n) < 0.05] = 0.0          # insert_hashtable drops values <= 0
    return vox, spot, val


def test_reference_table_keeps_each_positive_key_once(ref, tmp_path):
    vox, spot, val = _insertions()
    path = ref.ref_dij(vox, spot, val, 1 << 16, 7, (50, 20, 5), str(tmp_path))
    z = np.load(path)
    indptr, indices, data = z["indptr"], z["indices"], z["data"]
    assert list(z["shape"]) == [7, 5000] and z["format"] == b"csr"
    got = {}
    for s in range(7):
        for v, d in zip(indices[indptr[s]:indptr[s + 1]], data[indptr[s]:indptr[s + 1]]):
            assert (s, int(v)) not in got
            got[(s, int(v))] = d
    expect = {}
    for v, s, d in zip(vox, spot, val):
        if d > 0:
            expect[(int(s), int(v))] = expect.get((int(s), int(v)), 0.0) + d
    assert got.keys() == expect.keys()
    for k, d in expect.items():
        assert abs(got[k] - d) <= 1e-12 * d


def _members(path):
    """Raw zip members: name -> (local header, data bytes, central record)."""
    raw = open(path, "rb").read()
    eocd = raw.rfind(b"PK\x05\x06")
    n, cd_size, cd_off = struct.unpack("<HII", raw[eocd + 10:eocd + 20])
    out, p = {}, cd_off
    for _ in range(n):
        (csize, usize, nlen, xlen, clen) = struct.unpack("<IIHHH", raw[p + 20:p + 34])
        off = struct.unpack("<I", raw[p + 42:p + 46])[0]
        name = raw[p + 46:p + 46 + nlen].decode()
        cent = raw[p:p + 46 + nlen + xlen + clen]
        lnlen, lxlen = struct.unpack("<HH", raw[off + 26:off + 30])
        local = raw[off:off + 30 + lnlen + lxlen]
        data = raw[off + len(local):off + len(local) + csize]
        out[name] = (local, data, cent)
        p += len(cent)
    return out


def test_host_writer_matches_the_reference_writer_byte_for_byte(ref, tmp_path):
    vox, spot, val = _insertions(seed=4)
    ref_path = ref.ref_dij(vox, spot, val, 1 << 16, 7, (50, 20, 5), str(tmp_path), scale=2.5)
    z = np.load(ref_path)
    bins = {k: tmp_path / f"{k}.bin" for k in ("indices", "indptr", "data")}
    for k, p in bins.items():
        z[k].tofile(p)
    src = tmp_path / "w.cpp"
    src.write_text(r'''
#include "mqi_host.hpp"
#include <fstream>
#include <iterator>
static std::vector<char> slurp(const char* p) {
    std::ifstream f(p, std::ios::binary);
    return std::vector<char>(std::istreambuf_iterator<char>(f), {});
}
int main(int, char** argv) {
    const auto ind = slurp(argv[1]), ptr = slurp(argv[2]), dat = slurp(argv[3]);
    const uint32_t shape[2] = {(uint32_t) std::stoul(argv[4]), (uint32_t) std::stoul(argv[5])};
    const std::string n1 = "(" + std::to_string(ptr.size() / 4) + ",)", n2 = "(" + std::to_string(ind.size() / 4) + ",)";
    mqi_host::write_npz(argv[6], {{"indices", "<u4", n2, ind.data(), ind.size()},
                                  {"indptr", "<u4", n1, ptr.data(), ptr.size()},
                                  {"shape", "<u4", "(2,)", shape, sizeof(shape)},
                                  {"data", "<f8", n2, dat.data(), dat.size()},
                                  {"format", "|S3", "()", "csr", 3}});
    return 0;
}
''')
    exe = tmp_path / "w"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT}/include", f"-I{ROOT}/moquimc_gb300/host", str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    ours = tmp_path / "ours.npz"
    subprocess.run([str(exe), str(bins["indices"]), str(bins["indptr"]), str(bins["data"]), "7", "5000", str(ours)],
                   check=True)
    a, b = _members(ref_path), _members(str(ours))
    assert list(a) == list(b) == ["indices.npy", "indptr.npy", "shape.npy", "data.npy", "format.npy"]
    for name in ("indices.npy", "indptr.npy", "shape.npy", "data.npy"):
        assert a[name][0] == b[name][0], name          # local header (CRC and sizes included)
        assert a[name][1] == b[name][1], name          # .npy header and payload
        assert a[name][2] == b[name][2], name          # central directory record (offset included)
    la, lb = a["format.npy"], b["format.npy"]
    hdr = lb[1][:-3]
    assert la[1][:len(hdr)] == hdr and la[1][len(hdr):len(hdr) + 3] == b"csr" == lb[1][-3:]
    assert len(la[1]) - len(hdr) == 96                 # the reference's sizeof(std::string) x 3 bytes
    m = np.load(ours)
    assert m["format"] == b"csr" and (m["data"] == z["data"]).all()


def test_volume_writers_match_the_reference_writers_byte_for_byte(ref, tmp_path):
    """mqi_host::write_outputs (the host drivers' raw / mhd / mha) against the reference's own
    save_to_bin / save_to_mhd / save_to_mha (moqui/base/mqi_io.hpp:166-183, 493-583) on the same
    volume, grid and scale: identical files."""
    src = tmp_path / "vol.cpp"
    src.write_text(r'''
#include <fstream>
#include <moqui/base/mqi_node.hpp>
#include <moqui/base/mqi_io.hpp>
#include "mqi_host.hpp"
#include <random>
int main(int, char** argv) {
    const std::string ref = argv[1], ours = argv[2];
    const int nx = 7, ny = 5, nz = 9;
    std::vector<float> xe(nx + 1), ye(ny + 1), ze(nz + 1);
    for (int i = 0; i <= nx; ++i) xe[i] = -12.25f + 0.98f * i;
    for (int i = 0; i <= ny; ++i) ye[i] = 3.5f + 1.5f * i;
    for (int i = 0; i <= nz; ++i) ze[i] = -200.0f + 2.0f * i;
    std::mt19937_64 g(5);
    std::uniform_real_distribution<double> u(0.0, 1e-3);
    std::vector<double> d(nx * ny * nz);
    for (double& x : d) x = u(g);
    mqi::node_t<float> node;
    node.geo = new mqi::grid3d<mqi::density_t, float>(xe.data(), nx + 1, ye.data(), ny + 1, ze.data(), nz + 1);
    const float scale = 2.5f;
    mqi::io::save_to_bin<double>(d.data(), scale, ref, "v_bin", (uint32_t) d.size());
    mqi::io::save_to_mhd<float>(&node, d.data(), scale, ref, "v_mhd", (uint32_t) d.size());
    mqi::io::save_to_mha<float>(&node, d.data(), scale, ref, "v_mha", (uint32_t) d.size());
    mqi_host::write_outputs(ours, "v_bin", "raw", d, scale, xe, ye, ze);
    mqi_host::write_outputs(ours, "v_mhd", "mhd", d, scale, xe, ye, ze);
    mqi_host::write_outputs(ours, "v_mha", "mha", d, scale, xe, ye, ze);
    return 0;
}
''')
    exe = tmp_path / "vol"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-w", f"-I{ROOT}/oracle/_ref/src", f"-I{ROOT}/include",
                        f"-I{ROOT}/moquimc_gb300/host", str(src), "-o", str(exe), "-lz"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    a, b = tmp_path / "ref", tmp_path / "ours"
    a.mkdir()
    b.mkdir()
    subprocess.run([str(exe), str(a), str(b)], check=True, capture_output=True)
    names = ["v_bin.raw", "v_mhd.mhd", "v_mhd.raw", "v_mha.mha"]
    assert sorted(os.listdir(a)) == sorted(os.listdir(b)) == sorted(names)
    for n in names:
        assert (a / n).read_bytes() == (b / n).read_bytes(), n
