"""The moqui-side binding (moquimc_gb300/host/moqui_binding): a subclass of moqui's phantom_env that
keeps moqui's command line, world construction, host beam source and output writers and runs the
transport through the C ABI.  Built here with g++ against the staged reference headers and
include/mqi_gpu.h, linked to libmqigpu.so.  On the CPU: it compiles in moqui's debug and release
configurations, maps every callback moqui installs to the ABI's scorer enum (and rejects an unknown
one), and without a GPU fails cleanly in mqi_create after moqui's own initialisation."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIND = os.path.join(ROOT, "moquimc_gb300", "host", "moqui_binding")
REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src")


def build_binding(out_dir: str, debug: bool = True, main: str = None) -> str:
    from moquimc_gb300 import build

    build.build_library()
    exe = os.path.join(out_dir, "phantom_env_gb300" + ("_dbg" if debug else "_rel"))
    src = main or os.path.join(BIND, "phantom_env_gb300_main.cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-w", f"-I{REF_SRC}", f"-I{ROOT}/include", f"-I{BIND}", src, "-o", exe,
           f"-L{build.LIB_DIR}", "-lmqigpu", f"-Wl,-rpath,{build.LIB_DIR}", "-lz"]
    if debug:
        cmd.insert(3, "-D__PHYSICS_DEBUG__")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.fixture(scope="module")
def staged():
    if not os.path.isdir(os.path.join(REF_SRC, "moqui")):
        pytest.skip("the reference's staged sources are not present")
    return REF_SRC


@pytest.mark.parametrize("debug", [True, False])
def test_binding_compiles_against_the_reference(staged, tmp_path, debug):
    assert os.path.exists(build_binding(str(tmp_path), debug))


def test_scorer_callbacks_map_to_enums(staged, tmp_path):
    src = tmp_path / "map.cpp"
    src.write_text(r'''
#include <cstdio>
#include "mqi_gb300_binding.hpp"
template<typename R>
double user_callback(const mqi::track_t<R>&, const mqi::cnb_t&, mqi::grid3d<mqi::density_t, R>&, mqi::material_t<R>*&) {
    return 0.0;
}
int main() {
    const mqi::fp_compute_hit<float> fps[] = {
        mqi::energy_deposit<float>, mqi::energy_deposit_primary<float>, mqi::energy_deposit_secondary<float>,
        mqi::dose_to_water<float>, mqi::dose_to_water_square<float>, mqi::dose_to_medium<float>,
        mqi::LETd_weight1<float>, mqi::LETd_weight2<float>, mqi::LETt_weight1<float>, mqi::LETt_weight2<float>,
        user_callback<float>, nullptr };
    for (auto f : fps) {
        mqi::scorer<float> sc("s", 8, f);
        std::printf("%d\n", mqi_binding::scorer_type_of(&sc));
    }
    return 0;
}
''')
    exe = build_binding(str(tmp_path), True, str(src))
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    from moquimc_gb300 import capi

    assert [int(x) for x in out] == [capi.EDEP, capi.EDEP_PRIMARY, capi.EDEP_SECONDARY, capi.DOSE_W, capi.DOSE_W2,
                                     capi.DOSE_M, capi.LETD_NUM, capi.LETD_DEN, capi.LETT_NUM, capi.LETT_DEN,
                                     capi.MQI_ERR_UNSUPPORTED, capi.MQI_ERR_UNSUPPORTED]


def test_binding_without_a_gpu_fails_cleanly(staged, tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np

    exe = build_binding(str(tmp_path), True)
    ph = tmp_path / "ph.raw"
    np.zeros((4, 4, 4), np.int16).tofile(ph)
    r = subprocess.run([exe, "--lxyz", "10", "10", "10", "--pxyz", "0", "0", "-5", "--nxyz", "4", "4", "4",
                        "--spot_energy", "100", "0", "--spot_position", "0", "0", "0.5", "--spot_size", "1", "1",
                        "--histories", "10", "--phantom_path", str(ph), "--output_prefix", str(tmp_path),
                        "--random_seed", "3"], capture_output=True, text=True)
    assert r.returncode == 1 and "mqi_create" in r.stderr, (r.returncode, r.stderr[-500:])
