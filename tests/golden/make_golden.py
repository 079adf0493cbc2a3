#!/usr/bin/env python3
"""Generate the golden fixtures of the parity tests from the reference's own CPU build.

The reference ships no tests, golden vectors or known answers, so its CPU path -- compiled from the
reference headers by oracle/build_oracle.py -- is run here to produce them:

* ``raywalk.npz``   voxel index sequences and exit distances (as float bits) along seeded rays
                    through two grids (the phantom example's grid and a 0.98 x 0.98 x 2 mm CT-like grid
                    with a non-integer origin), including rays started on voxel edges, with zero or tiny
                    direction components, and from outside the grid.
* ``physics.npz``   the deterministic physics functions on fixed input grids (cross sections, stopping
                    power, relativistic quantities, SPR, radiation length, straggling variance) and
                    HU -> density for every HU in [-1100, 3100].
* ``dose_c1.npz``   the phantom example (200x200x350 water, 200 MeV, +-30 mm square, debug physics):
                    per-batch laterally integrated depth dose and a coarse 3-D dose over 8 batches of
                    12500 histories (1e5 in total).
* ``dose_c2.npz``   the slab phantom (256^3, lung + bone, 150 MeV Gaussian sigma 4 mm, release
                    physics): the same statistics over 8 batches of 12500 histories.
* ``dose_c3.npz``   three Gaussian spots (sigma 4 mm) of different energies and positions on the
                    synthetic CT (512x512x200, 0.98x0.98x2 mm, release physics): per-batch
                    laterally integrated depth dose and a coarse dose in a 49x49-voxel column around
                    each spot, 8 batches of 12500 histories per spot.
* ``vertices.npz``  phantom_env's host beam source (coordinate_transform + phsp_6d_uniform or
                    phsp_6d + const_1d, std::default_random_engine) for a few seeds, spot shapes and
                    gantry/couch angles: the vertices the C++ host driver must reproduce bit for bit.

Run from the repository root: ``python tests/golden/make_golden.py``.  It needs the reference sources
(to stage and build the CPU oracle) and takes about a minute on 8 cores.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mqo  # noqa: E402
from moquimc_gb300 import phantom as ph  # noqa: E402
from moquimc_gb300 import workloads  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def ray_set(rng, lo, hi, edges, n):
    """Seeded rays: random interior/exterior starts, some snapped to edges, some axis-aligned or
    with tiny direction components."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    span = hi - lo
    pos = lo - 0.1 * span + rng.random((n, 3)) * 1.2 * span
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    k = n // 8
    for ax in range(3):
        idx = rng.integers(0, n, k)
        pos[idx, ax] = rng.choice(edges[ax], k)          # exactly on an edge
    idx = rng.integers(0, n, k)
    d[idx, 0] = 0.0                                       # zero component
    idx = rng.integers(0, n, k)
    d[idx, 1] = rng.choice([1e-4, -2e-4, 3e-4], k)        # below the 1e-7 square threshold
    idx = rng.integers(0, n, k // 2)
    d[idx] = [0.0, 0.0, -1.0]                             # the beam direction
    idx = rng.integers(0, n, k // 2)
    d[idx] = [0.0, 0.0, 1.0]
    pos = pos.astype(np.float32)
    d = d.astype(np.float32)
    return np.concatenate([pos, d], axis=1)


def make_raywalk():
    rng = np.random.default_rng(20261203)
    grids = {
        "phantom": ((-50.0, 50.0, -50.0, 50.0, -350.0, 0.0), (200, 200, 350), 1200),
        "ct": ((-250.88, 250.88, -200.9, 300.86, -210.0, 190.0), (512, 512, 200), 800),
    }
    out = {}
    for name, (bounds, n, nrays) in grids.items():
        edges = [ph.uniform_edges(bounds[2 * a], bounds[2 * a + 1], n[a]) for a in range(3)]
        rays = ray_set(rng, bounds[0::2], bounds[1::2], edges, nrays)
        max_steps = 4 * sum(n)
        off, cnb, dist, cells = mqo.ref_trace_rays(bounds, n, rays, max_steps)
        out[f"{name}_bounds"] = np.asarray(bounds, np.float32)
        out[f"{name}_n"] = np.asarray(n, np.int32)
        out[f"{name}_max_steps"] = np.int64(max_steps)
        out[f"{name}_rays"] = rays
        out[f"{name}_offsets"] = off
        out[f"{name}_cnb"] = cnb.astype(np.uint32)
        out[f"{name}_dist_bits"] = dist.view(np.uint32)
        print(name, "rays", len(rays), "entries", len(cnb))
    np.savez_compressed(os.path.join(OUT, "raywalk.npz"), **out)


def make_physics():
    import tempfile

    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "phys.bin")
        import subprocess

        out = {}
        for debug in (True, False):
            subprocess.run([mqo.ref_binary(debug), "physics", path], check=True, capture_output=True)
            names = ["energies", "rhos", "beta_sq", "gamma", "te_max", "et", "momentum", "cs_ion", "cs_pp", "cs_poe",
                     "cs_poi", "dedx", "spr", "x0", "straggling", "hu_rho"]
            vecs = mqo.read_vecs(path, [np.float32] * len(names))
            tag = "dbg" if debug else "rel"
            for nm, v in zip(names, vecs):
                if nm in ("spr", "x0", "straggling"):
                    out[f"{nm}_{tag}"] = v
                elif debug:
                    out[nm] = v
        out["hu"] = np.arange(-1100, 3101, dtype=np.int32)
    np.savez_compressed(os.path.join(OUT, "physics.npz"), **out)
    print("physics", {k: v.shape for k, v in out.items()})


def coarse(dose, nxyz, b):
    nx, ny, nz = nxyz
    d = dose.reshape(nz, ny, nx)
    return d.reshape(nz // b[2], b[2], ny // b[1], b[1], nx // b[0], b[0]).sum(axis=(1, 3, 5))


def make_dose(wl, fname, batches=8, each=12500, seed0=31000, coarse_bins=(10, 10, 10)):
    dose, recs, doses = mqo.ref_phantom_parallel(wl.physics_debug, wl.lxyz, wl.pxyz, wl.nxyz, wl.energy,
                                                 wl.spot_position, wl.spot_size, each, batches, wl.hu, seed0,
                                                 beam=wl.beam)
    idd = np.array([ph.depth_dose(d, wl.nxyz) for d in doses]) / each
    crs = np.array([coarse(d, wl.nxyz, coarse_bins) for d in doses]) / each
    secs = np.array([r["transport_seconds"] for r in recs])
    np.savez_compressed(os.path.join(OUT, fname), idd=idd, coarse=crs.astype(np.float64),
                        coarse_bins=np.asarray(coarse_bins), histories_per_batch=np.int64(each),
                        transport_seconds=secs, nxyz=np.asarray(wl.nxyz), physics_debug=np.int64(wl.physics_debug))
    r80 = ph.r80(idd.mean(0), wl.lxyz[2] / wl.nxyz[2])
    print(fname, "R80", r80, "per-core primaries/s", each / secs.mean())


C3_SPOTS = [(0.0, 0.0, 150.0), (-40.0, 30.0, 200.0), (60.0, -20.0, 110.0)]   # x, y (mm), energy (MeV)
C3_CROP = 24          # voxels either side of the spot's column
C3_BINS = (7, 7, 4)   # coarse bins of the 49 x 49 x 200 crop


def c3_crop(dose, wl, x, y):
    """The 49 x 49 voxel column around the spot (x, y), binned 7 x 7 x 4: shape (50, 7, 7)."""
    return ph.column_crop(dose, wl.lxyz, wl.nxyz, x, y, C3_CROP, C3_BINS)


def make_dose_c3(batches=8, each=12500, seed0=51000):
    wl = workloads.c3()
    out = {"spots": np.array(C3_SPOTS), "histories_per_batch": np.int64(each), "bins": np.array(C3_BINS),
           "crop": np.int64(C3_CROP)}
    for k, (x, y, e) in enumerate(C3_SPOTS):
        _, recs, doses = mqo.ref_phantom_parallel(False, wl.lxyz, wl.pxyz, wl.nxyz, e, (x, y, 195.0), (4.0, 4.0), each,
                                                  batches, wl.hu, seed0 + 100 * k, beam="gaussian")
        out[f"idd{k}"] = np.array([ph.depth_dose(d, wl.nxyz) for d in doses]) / each
        out[f"coarse{k}"] = np.array([c3_crop(d, wl, x, y) for d in doses]) / each
        out[f"seconds{k}"] = np.array([r["transport_seconds"] for r in recs])
        print("c3 spot", k, "R80", ph.r80(out[f"idd{k}"].mean(0), 2.0), "per-core primaries/s",
              each / out[f"seconds{k}"].mean(), flush=True)
    np.savez_compressed(os.path.join(OUT, "dose_c3.npz"), **out)


VERTEX_CASES = [
    # seed, gaussian, position, size, energy, angles (collimator, gantry, couch, iec2dicom)
    (1234, 0, (0.0, 0.0, 0.5), (30.0, 30.0), 200.0, (0.0, 0.0, 0.0, 0.0)),
    (7, 0, (1.0, 2.0, 3.0), (10.0, 5.0), 150.0, (10.0, 30.0, 5.0, 90.0)),
    (99, 1, (0.0, 0.0, 0.5), (4.0, 4.0), 150.0, (0.0, 45.0, 0.0, 0.0)),
]


def make_vertices(n=2000):
    import subprocess
    import tempfile

    out = {}
    for k, (seed, gaus, pos, size, e, ang) in enumerate(VERTEX_CASES):
        with tempfile.TemporaryDirectory() as td:
            f = os.path.join(td, "v.bin")
            cmd = [mqo.ref_binary(False), "vertices", f, str(n), str(seed), str(gaus), *map(str, pos), *map(str, size),
                   str(e), *map(str, ang)]
            subprocess.run(cmd, check=True, capture_output=True)
            out[f"case{k}"] = mqo.read_vecs(f, [np.float32])[0].reshape(-1, 7)
        out[f"args{k}"] = np.array([seed, gaus, *pos, *size, e, *ang], np.float64)
    np.savez_compressed(os.path.join(OUT, "vertices.npz"), **out)
    print("vertices", {k: v.shape for k, v in out.items()})


def main():
    if not mqo.ref_available():
        raise SystemExit("the reference CPU build is not available")
    which = sys.argv[1:] or ["raywalk", "physics", "dose_c1", "dose_c2", "dose_c3", "vertices"]
    if "raywalk" in which:
        make_raywalk()
    if "physics" in which:
        make_physics()
    if "dose_c1" in which:
        make_dose(workloads.c1(), "dose_c1.npz")
    if "dose_c2" in which:
        make_dose(workloads.c2(), "dose_c2.npz", seed0=41000, coarse_bins=(8, 8, 4))
    if "dose_c3" in which:
        make_dose_c3()
    if "vertices" in which:
        make_vertices()


if __name__ == "__main__":
    main()
