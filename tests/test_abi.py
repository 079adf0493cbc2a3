"""The C ABI library loads and exports every entry point include/mqi_gpu.h declares (no GPU work)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "mqi_gpu.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mqi_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for must in ("mqi_create", "mqi_transport", "mqi_get_tally", "mqi_set_vertices", "mqi_trace_rays"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(built_lib):
    from moquimc_gb300 import capi

    assert set(declared_functions()) <= set(capi.EXPORTS)


def test_version_string(built_lib):
    assert b"sm_103a" in built_lib.mqi_version()


def test_errors_are_status_codes_not_exits(built_lib):
    """Bad arguments come back as negative codes with a message (moqui calls exit() instead)."""
    lib = built_lib
    assert lib.mqi_create(0, None) == -1
    assert b"NULL" in lib.mqi_last_error(None)
    assert lib.mqi_transport(None, 0, 1, 0) == -1
    assert lib.mqi_set_physics(None, 1, 1) == -1


def test_create_without_device_fails_cleanly(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = built_lib.mqi_create(0, ctypes.byref(h))
    assert rc in (-1, -2)
    assert h.value is None
    assert built_lib.mqi_last_error(None)


def test_struct_layouts_match_the_header(tmp_path):
    """The numpy dtypes the binding passes across the ABI have the C structs' offsets and sizes."""
    import shutil
    import subprocess

    import numpy as np

    from moquimc_gb300 import capi

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "mqi_gpu.h"\n'
        "#define O(t, f) printf(\"%zu \", offsetof(t, f))\n"
        "int main(void) {\n"
        " O(mqi_spot, energy); O(mqi_spot, energy_sigma); O(mqi_spot, mean); O(mqi_spot, sigma);\n"
        " O(mqi_spot, corr); O(mqi_spot, rot); O(mqi_spot, trans); O(mqi_spot, histories);\n"
        " printf(\"%zu %zu \", sizeof(mqi_spot), sizeof(mqi_vertex));\n"
        " printf(\"%zu %zu\\n\", offsetof(mqi_tune_result, histories_per_s), sizeof(mqi_tune_result));\n return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    d = capi.SPOT_DTYPE
    assert got[:8] == [d.fields[n][1] for n in d.names]
    assert got[8] == d.itemsize
    assert got[9] == capi.VERTEX_DTYPE.itemsize == 28
    assert got[10] == capi.TUNE_DTYPE.fields["histories_per_s"][1] and got[11] == capi.TUNE_DTYPE.itemsize
    assert np.dtype(capi.SPOT_DTYPE).names[-1] == "histories"
