#!/usr/bin/env python3
"""Time the reference's own CUDA kernel on this GPU (test infrastructure; measurement only).

Runs oracle/ref_gpu_driver.cu -- moqui's transport_particles_patient<float> compiled for sm_103a
from the staged reference headers -- on the phantom-example water box (200x200x350 voxels, 200 MeV
uniform +-30 mm spot, debug physics, the example's own build) and on the heterogeneous slab
phantom (256^3, 150 MeV Gaussian sigma 4 mm, release physics as the benchmark runs it), and
prints one JSON line per run: primaries/s = histories / CUDA-event kernel time.

Usage: python oracle/time_ref_gpu.py [--c1 100000] [--c2 1000000] [--repeats 2] [--out <dir>]
"""
import argparse
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

import mqo  # noqa: E402

from moquimc_gb300 import workloads  # noqa: E402


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--c1", type=int, default=100_000)
    ap.add_argument("--c2", type=int, default=1_000_000)
    ap.add_argument("--repeats", type=int, default=2)
    ap.add_argument("--out", default="")
    args = ap.parse_args()
    out = args.out or tempfile.mkdtemp(prefix="mqi_refgpu_")
    for wl, n in ((workloads.c1(args.c1), args.c1), (workloads.c2(args.c2), args.c2)):
        if n <= 0:
            continue
        wdir = os.path.join(out, wl.name)
        os.makedirs(wdir, exist_ok=True)
        ph = os.path.join(wdir, "phantom.raw")
        wl.hu.astype("int16").tofile(ph)
        for r in range(args.repeats):
            rdir = os.path.join(wdir, f"r{r}")
            os.makedirs(rdir, exist_ok=True)
            _, rec = mqo.ref_gpu_phantom(wl.physics_debug, wl.lxyz, wl.pxyz, wl.nxyz, wl.energy, wl.spot_position,
                                         wl.spot_size, n, None, 1 + r, wl.beam, workdir=rdir, phantom_path=ph)
            rec.update(workload=wl.name, repeat=r, primaries_per_s=rec["histories"] / (rec["kernel_ms"] * 1e-3))
            print(json.dumps(rec), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
