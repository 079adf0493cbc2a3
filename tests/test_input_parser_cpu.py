"""The treatment-planning drivers' input-file reader against moqui's own (mqi::file_parser,
moqui/base/mqi_file_handler.hpp:220-420, compiled by the oracle recipe from the staged reference
headers into oracle/_ref/bin/ref_parser).  Three readers answer the same queries on the same files:
moqui's, the C++ driver's (mqi_host::InputFile, moquimc_gb300/host/mqi_host.hpp, compiled here into
a small harness) and the Python environment's (moquimc_gb300.tps.InputFile).  The files exercise
the reader's rules: '#' comments (whole lines, indented, trailing, without a space before them),
white space (tabs, CR of CRLF files, form feed and vertical tab), case-insensitive keys, the first
matching line winning, a tab instead of the space after a key, keys without a value, numbers as
atof / atoi read them (prefixes, hexadecimal floats, inf, -0), booleans ("true" in any case or a
non-zero integer), defaults of missing keys written with std::to_string first (so a float default
keeps six decimals), and comma-separated lists.

Where moqui's reader throws (a line of white space only; a value of white space only; an empty
item in a comma-separated list) the drivers read on; those files are checked separately.

The mask files of ScoringMask / StatROIMaskFilename are checked the same way against moqui's
mask_reader (read_mask_files, mask_to_roi): the summed mask and its CONTOUR runs."""
import os
import subprocess

import numpy as np
import pytest

from moquimc_gb300 import tps

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <string>
#include "mqi_host.hpp"
int main(int argc, char** argv) {
    mqi_host::InputFile p(argv[1]);
    for (int i = 2; i < argc; ++i) {
        const std::string q = argv[i];
        const size_t a = q.find(':', 2);
        const std::string key = q.substr(2, a - 2), dflt = q.substr(a + 1);
        switch (q[0]) {
        case 's': std::printf("%s\n", p.get_string(key, dflt).c_str()); break;
        case 'f': std::printf("%.9g\n", p.get_float(key, (float) std::atof(dflt.c_str()))); break;
        case 'i': std::printf("%d\n", p.get_int(key, std::atoi(dflt.c_str()))); break;
        case 'b': std::printf("%d\n", (int) p.get_bool(key, std::atoi(dflt.c_str()) != 0)); break;
        case 'v': {
            const auto v = p.get_vector(key, ',');
            std::string out;
            for (size_t k = 0; k < v.size(); ++k) out += (k ? "|" : "") + v[k];
            std::printf("%s\n", out.c_str());
            break;
        }
        }
    }
    return 0;
}
"""

CASES = {
    "keys": ("GPUID 0\nRandomSeed -1932780356\nUseAbsolutePath true\nScorer Dose, LETd ,TrackLength  \n"
             "SimulationType perSpot\nParticlesPerHistory 1000\nRBE 1.1\nNumberOfFraction 30\n"
             "OutputDir /tmp/some dir/with spaces\nOutputFormat mhd\n",
             ["s:OutputDir:x", "v:Scorer:", "i:RandomSeed:0", "b:UseAbsolutePath:0", "f:RBE:1.1",
              "i:NumberOfFraction:1", "f:ParticlesPerHistory:-1", "s:simulationtype:perBeam", "s:OUTPUTFORMAT:raw",
              "s:Missing:dflt", "f:Missing:1e-7", "f:Missing:2.5", "f:Missing:-1", "i:Missing:-1", "b:Missing:1",
              "b:Missing:0", "v:Missing:"]),
    "comments_and_white_space": ("# leading comment\n   # indented comment\nMachine PBS:model.txt   # trailing\n"
                                 "\tRBE 1.2\t\nXShift 3.5#no space before the hash\nYShift  -2.25  \nZShift 1e-3\n"
                                 "DensityScaling .965\nStatThreshold 5.\nStoppingCriteria +2\nBeamNumbers 2, 1,3\n"
                                 "OverwriteResults TRUE\r\n\fStatROI 3\v\nCalibration default\r\n",
                                 ["s:Machine:", "f:RBE:0", "f:XShift:0", "f:YShift:0", "f:ZShift:0",
                                  "f:DensityScaling:1", "f:StatThreshold:0", "f:StoppingCriteria:-1", "v:BeamNumbers:",
                                  "b:OverwriteResults:0", "i:StatROI:0", "s:Calibration:x"]),
    "first_match_and_odd_values": ("RBE 1.3\nrbe 1.4\nRandomSeed 12abc\nUnitWeights 3.9\nFlag yes\nFlag2 FALSE\n"
                                   "Flag3 2\nHex 0x1p4\nBig 1e39\nInf inf\nTabKey\t5\nEmpty\nNeg -0\n"
                                   "Spaced   value with   inner  spaces   \n",
                                   ["f:RBE:0", "i:RandomSeed:0", "i:UnitWeights:0", "b:Flag:1", "b:Flag2:1",
                                    "b:Flag3:0", "f:Hex:0", "f:Big:0", "f:Inf:0", "s:TabKey:dflt", "s:Empty:dflt",
                                    "f:Neg:1", "s:Spaced:x", "i:Spaced:7"]),
}


@pytest.fixture(scope="module")
def ref_parser(oracle):
    if not oracle.ref_available():
        pytest.skip("the reference's staged sources are not present")
    import build_oracle

    exe = build_oracle.ref_parser_binary()
    if not os.path.exists(exe):
        build_oracle.build_reference()
    if not os.path.exists(exe):
        pytest.skip("the staged reference has no input-file reader")
    return exe


@pytest.fixture(scope="module")
def host_parser(tmp_path_factory):
    d = tmp_path_factory.mktemp("harness")
    src, exe = os.path.join(d, "h.cpp"), os.path.join(d, "h")
    with open(src, "w") as f:
        f.write(HARNESS)
    r = subprocess.run(["g++", "-std=c++17", "-O1", f"-I{os.path.join(ROOT, 'moquimc_gb300', 'host')}",
                        f"-I{os.path.join(ROOT, 'include')}", src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _python(path, queries):
    p = tps.InputFile.load(path)
    out = []
    for q in queries:
        t, rest = q[0], q[2:]
        key, dflt = rest.split(":", 1)
        if t == "s":
            out.append(p.get_string(key, dflt))
        elif t == "f":
            out.append("%.9g" % np.float32(p.get_float(key, float(np.float32(float(dflt))))))
        elif t == "i":
            out.append(str(p.get_int(key, int(dflt))))
        elif t == "b":
            out.append(str(int(p.get_bool(key, int(dflt) != 0))))
        else:
            out.append("|".join(p.get_string_vector(key, ",")))
    return out


def _run(exe, path, queries):
    r = subprocess.run([exe, path, *queries], capture_output=True, text=True)
    return r.returncode, r.stdout.split("\n")[:len(queries)], r.stderr


@pytest.mark.parametrize("case", sorted(CASES))
def test_drivers_read_input_files_as_moqui_does(case, ref_parser, host_parser, tmp_path):
    text, queries = CASES[case]
    path = os.path.join(tmp_path, "in.txt")
    with open(path, "w", newline="") as f:
        f.write(text)
    rc, ref, err = _run(ref_parser, path, queries)
    assert rc == 0, err
    rc, cpp, err = _run(host_parser, path, queries)
    assert rc == 0, err
    py = _python(path, queries)
    for q, a, b, c in zip(queries, ref, cpp, py):
        assert a == b == c, (case, q, a, b, c)


@pytest.mark.parametrize("text,expect", [("RBE 1.3\n   \nXShift 2\n", "2"),
                                         ("RBE 1.3\nXShift  #only a comment after the key\n", ""),
                                         ("RBE 1.3\nXShift Dose, ,LETd,\n", "Dose|LETd")])
def test_white_space_moqui_throws_on_is_read_on(text, expect, ref_parser, host_parser, tmp_path):
    """moqui's trim_copy calls substr(npos) on a string of white space only (or an empty one), so its
    reader throws on a line of white space only, on a key whose value is white space only, and on
    an empty item of a comma-separated list; the drivers skip the line, read the value as "" and
    skip the empty items, and read the other keys."""
    path = os.path.join(tmp_path, "in.txt")
    with open(path, "w") as f:
        f.write(text)
    queries = ["f:RBE:0", ("v" if "," in text else "s") + ":XShift:x"]
    rc, _, err = _run(ref_parser, path, queries)
    assert rc == 3 and err
    expect = ["1.29999995", expect]
    rc, cpp, err = _run(host_parser, path, queries)
    assert rc == 0 and cpp == expect, (cpp, err)
    assert _python(path, queries) == expect


# ---- masks: mask_reader::read_mask_files + mask_to_roi (moqui/base/mqi_file_handler.hpp:13-218)

def _write_mha(path, mask, dims, style=0):
    nx, ny, nz = dims
    keys = [("ObjectType", "Image"), ("NDims", "3"), ("BinaryData", "True"), ("BinaryDataByteOrderMSB", "False"),
            ("CompressedData", "False"), ("TransformMatrix", "1 0 0 0 1 0 0 0 1"), ("Offset", "-10 -20 5.5"),
            ("CenterOfRotation", "0 0 0"), ("AnatomicalOrientation", "RAI"), ("ElementSpacing", "1 1 2"),
            ("DimSize", f"{nx} {ny} {nz}"), ("ElementType", "MET_UCHAR"), ("ElementDataFile", "LOCAL")]
    if style == 1:   # other spacing around '=' and other key case, as MHA writers vary
        lines = [f"{k.lower() if i % 2 else k}={v}" if i % 3 else f"  {k}  =   {v}  " for i, (k, v) in enumerate(keys)]
    else:
        lines = [f"{k} = {v}" for k, v in keys]
    with open(path, "wb") as f:
        f.write(("\n".join(lines) + "\n").encode() + np.asarray(mask, np.uint8).tobytes())


def _ref_runs(exe, dims, files):
    r = subprocess.run([exe, "--mask", *map(str, dims), *files], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [ln.split() for ln in r.stdout.splitlines() if ln.startswith(("roi ", "run "))]
    assert lines[0][0] == "roi" and int(lines[0][1]) == len(lines) - 1
    return [tuple(x[1:]) for x in lines[1:]]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mask_runs_match_moqui(seed, ref_parser, tmp_path):
    """Two or three random masks (overlaps sum to 2, which continues a run but does not start one),
    written with varied header formatting: the summed mask and its CONTOUR runs (start, stride,
    accumulated stride) equal moqui's, run for run."""
    rng = np.random.default_rng(seed)
    dims = (30, 20, 10)
    n = int(np.prod(dims))
    files, total = [], np.zeros(n, np.int64)
    for k in range(2 + seed % 2):
        m = np.zeros(n, np.uint8)
        for _ in range(40):   # boxes of ones, so that runs of many lengths occur
            a = rng.integers(0, n - 1)
            m[a:a + rng.integers(1, 60)] = 1
        m[-1] = 0             # every run closes inside the volume
        path = os.path.join(tmp_path, f"m{k}.mha")
        _write_mha(path, m, dims, style=k % 2)
        files.append(path)
        total += m
    ref = _ref_runs(ref_parser, dims, files)
    summed = sum(tps.read_mask_mha(f).astype(np.int64) for f in files)
    np.testing.assert_array_equal(summed, total)
    start, stride, acc = tps.mask_to_contour(summed)
    assert [tuple(map(str, t)) for t in zip(start, stride, acc)] == ref
    assert (summed == 2).any()


def test_mask_run_open_at_the_end(ref_parser, tmp_path):
    """A run that reaches the last voxel: moqui starts it and leaves its stride unset; here it is
    closed at the end of the volume."""
    dims = (4, 3, 2)
    m = np.zeros(24, np.uint8)
    m[2:5] = 1
    m[20:] = 1
    path = os.path.join(tmp_path, "m.mha")
    _write_mha(path, m, dims)
    ref = _ref_runs(ref_parser, dims, [path])
    assert ref == [("2", "3", "3"), ("20", "open")]
    start, stride, acc = tps.mask_to_contour(tps.read_mask_mha(path))
    assert list(start) == [2, 20] and list(stride) == [3, 4] and list(acc) == [3, 7]
