"""Synthetic workloads of the benchmark configurations (seeded; no patient data exists).

* ``c1``: moqui's phantom example -- a 100x100x350 mm water box (HU 0) of 200x200x350 voxels,
  one 200 MeV spot with a uniform +-30 mm square profile, 1e5 histories, debug physics (the
  example is built with -D__PHYSICS_DEBUG__).
* ``c2``: a 256^3 phantom of 1 mm voxels centred at (0, 0, -128): water (HU 0) with a 30 mm lung
  slab (HU -700) and a 15 mm bone slab (HU 1200) at depths drawn from numpy's default_rng(2) in
  40-180 mm, full lateral extent; one 150 MeV Gaussian spot (sigma 4 mm), 1e6 histories.
* ``c3``: a synthetic CT of 512x512x200 voxels at 0.98x0.98x2 mm centred at the origin: an
  ellipsoidal body (semi-axes 180/120/180 mm on x/y/z) whose HU is white noise from
  default_rng(4), Gaussian-smoothed (sigma 5 mm) and rescaled to mean 40 and s.d. 150, clipped to
  [-1000, 1500], in air (HU -1000); a plan of 2000 Gaussian spots (sigma 4 mm, no divergence) on a
  5 mm grid (50 on x by 40 on y) entering at z = 195 mm along -z, energies uniform in 70-230 MeV
  (default_rng(5)), history counts lognormal (default_rng(6)) with the 1st-99th percentiles at
  1e3-1e5, clipped to that range.
* ``c4``: the c3 CT and plan x 21 robust scenarios: setup shifts 0, +-3 mm on x, y and z, each with
  DensityScaling 1, 1.035 and 0.965.
* ``c5``: the c3 Dij with a 60 mm spherical target at the body centre and a 20 mm spherical organ
  placed by default_rng(7) outside it; finite differences on 64 spots drawn by default_rng(8).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import phantom as ph


@dataclass
class Workload:
    name: str
    lxyz: tuple
    pxyz: tuple
    nxyz: tuple
    hu: np.ndarray            # int16, [nz][ny][nx]
    energy: float
    beam: str                 # "uniform" (half-width) or "gaussian" (sigma)
    spot_size: tuple
    spot_position: tuple
    histories: int
    physics_debug: bool
    meta: dict = field(default_factory=dict)

    def edges(self):
        return ph.phantom_box_edges(self.lxyz, self.pxyz, self.nxyz)

    def vertices(self, n: int, seed: int) -> np.ndarray:
        rng = np.random.default_rng(seed)
        if self.beam == "uniform":
            return ph.uniform_spot_vertices(n, rng, self.energy, self.spot_position, self.spot_size)
        return ph.gaussian_spot_vertices(n, rng, self.energy, self.spot_position, self.spot_size)


def c1(histories: int = 100_000) -> Workload:
    nxyz = (200, 200, 350)
    return Workload("c1_water_phantom_200MeV", (100.0, 100.0, 350.0), (0.0, 0.0, -175.0), nxyz,
                    np.zeros(nxyz[::-1], np.int16), 200.0, "uniform", (30.0, 30.0), (0.0, 0.0, 0.5), histories,
                    True)


def slab_depths(seed: int = 2):
    """Start depths (mm from the entrance) of the lung (30 mm) and bone (15 mm) slabs: both inside
    40-180 mm and not overlapping."""
    rng = np.random.default_rng(seed)
    while True:
        lung = float(rng.uniform(40.0, 180.0 - 30.0))
        bone = float(rng.uniform(40.0, 180.0 - 15.0))
        if lung + 30.0 <= bone or bone + 15.0 <= lung:
            return int(round(lung)), int(round(bone))


def c2(histories: int = 1_000_000, physics_debug: bool = False) -> Workload:
    n = 256
    hu = np.zeros((n, n, n), np.int16)
    lung, bone = slab_depths(2)
    # depth d mm occupies z index n-1-d (the beam enters at z = 0 and travels along -z)
    for start, thick, val in ((lung, 30, -700), (bone, 15, 1200)):
        for d in range(start, start + thick):
            hu[n - 1 - d, :, :] = val
    return Workload("c2_slab_phantom_150MeV", (256.0, 256.0, 256.0), (0.0, 0.0, -128.0), (n, n, n), hu, 150.0,
                    "gaussian", (4.0, 4.0), (0.0, 0.0, 0.5), histories, physics_debug,
                    {"lung_depth_mm": lung, "bone_depth_mm": bone})


def ct_hu(nxyz=(512, 512, 200), dxyz=(0.98, 0.98, 2.0), semi=(180.0, 120.0, 180.0), mean=40.0, sd=150.0,
          smooth_mm=5.0, seed=4) -> np.ndarray:
    """int16 HU [nz][ny][nx] of the synthetic CT body.  The random field is drawn and smoothed only
    on the body's bounding box (the air outside does not use it)."""
    from scipy.ndimage import gaussian_filter

    nx, ny, nz = nxyz
    centres = [(np.arange(n, dtype=np.float64) + 0.5) * d - 0.5 * n * d for n, d in zip(nxyz, dxyz)]
    box = [np.where(np.abs(c) <= a + d)[0] for c, a, d in zip(centres, semi, dxyz)]
    sl = tuple(slice(int(b[0]), int(b[-1]) + 1) for b in box)          # x, y, z ranges
    rng = np.random.default_rng(seed)
    shape = (sl[2].stop - sl[2].start, sl[1].stop - sl[1].start, sl[0].stop - sl[0].start)
    field = rng.standard_normal(shape, dtype=np.float32)
    field = gaussian_filter(field, sigma=(smooth_mm / dxyz[2], smooth_mm / dxyz[1], smooth_mm / dxyz[0]),
                            mode="reflect", truncate=3.0)
    field = (field - field.mean()) / field.std()
    hu_box = np.clip(np.rint(mean + sd * field), -1000, 1500).astype(np.int16)
    cz, cy, cx = np.meshgrid(centres[2][sl[2]], centres[1][sl[1]], centres[0][sl[0]], indexing="ij")
    inside = (cx / semi[0]) ** 2 + (cy / semi[1]) ** 2 + (cz / semi[2]) ** 2 <= 1.0
    hu = np.full((nz, ny, nx), -1000, np.int16)
    hu[sl[2], sl[1], sl[0]] = np.where(inside, hu_box, np.int16(-1000))
    return hu


def spot_plan(n_x=50, n_y=40, pitch=5.0, z0=195.0, sigma=4.0, e_range=(70.0, 230.0), h_range=(1e3, 1e5),
              seeds=(5, 6)) -> np.ndarray:
    """Spots on a pitch grid centred on the beam axis, beam along -z (identity beam-to-world
    transform), energies uniform in e_range, history counts lognormal with the 1st and 99th
    percentiles at h_range, clipped to it."""
    from .capi import SPOT_DTYPE

    n = n_x * n_y
    sp = np.zeros(n, SPOT_DTYPE)
    gx = (np.arange(n_x) - 0.5 * (n_x - 1)) * pitch
    gy = (np.arange(n_y) - 0.5 * (n_y - 1)) * pitch
    X, Y = np.meshgrid(gx, gy, indexing="xy")
    sp["energy"] = np.random.default_rng(seeds[0]).uniform(*e_range, n).astype(np.float32)
    sp["mean"][:, 0] = X.ravel()
    sp["mean"][:, 1] = Y.ravel()
    sp["mean"][:, 2] = z0
    sp["sigma"][:, 0] = sigma
    sp["sigma"][:, 1] = sigma
    sp["rot"] = np.eye(3, dtype=np.float32).ravel()
    lo, hi = np.log(h_range[0]), np.log(h_range[1])
    z99 = 2.3263478740408408                                   # standard normal 99th percentile
    h = np.exp(np.random.default_rng(seeds[1]).normal(0.5 * (lo + hi), 0.5 * (hi - lo) / z99, n))
    sp["histories"] = np.clip(np.rint(h), h_range[0], h_range[1]).astype(np.uint64)
    return sp


@dataclass
class PlanWorkload:
    name: str
    lxyz: tuple
    pxyz: tuple
    nxyz: tuple
    hu: np.ndarray
    spots: np.ndarray
    physics_debug: bool
    meta: dict = field(default_factory=dict)

    def edges(self):
        return ph.phantom_box_edges(self.lxyz, self.pxyz, self.nxyz)

    @property
    def histories(self) -> int:
        return int(self.spots["histories"].sum())


_CT_CACHE: dict = {}


def c3(physics_debug: bool = False) -> PlanWorkload:
    nxyz = (512, 512, 200)
    key = ("c3", nxyz)
    if key not in _CT_CACHE:
        _CT_CACHE[key] = ct_hu(nxyz)
    hu = _CT_CACHE[key]
    lxyz = (float(np.float32(512 * 0.98)), float(np.float32(512 * 0.98)), 400.0)
    return PlanWorkload("c3_synthetic_ct_2000_spots", lxyz, (0.0, 0.0, 0.0), nxyz, hu, spot_plan(), physics_debug)


def c4_scenarios():
    """The 21 robust scenarios: (shift mm, density scale)."""
    shifts = [(0.0, 0.0, 0.0)] + [tuple(sg * 3.0 if i == ax else 0.0 for i in range(3)) for ax in range(3)
                                  for sg in (1, -1)]
    return [(sh, sc) for sh in shifts for sc in (1.0, 1.035, 0.965)]


def scenario_edges(wl, shift):
    """Edges of the shifted CT: the origin moves by the shift, then the edges are formed from it
    (tps_env, mqi_tps_env.hpp:475-477 and 507-514)."""
    p = tuple(np.float32(a) + np.float32(b) for a, b in zip(wl.pxyz, shift))
    return ph.phantom_box_edges(wl.lxyz, p, wl.nxyz)


def c5_structures(wl, target_radius=60.0, organ_radius=20.0, seed=7):
    """Boolean voxel masks (flat, x fastest) of the spherical target at the body centre and of the
    organ placed by default_rng(seed) outside the target and inside the body."""
    rng = np.random.default_rng(seed)
    semi = np.array([180.0, 120.0, 180.0])
    while True:
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        c = d * rng.uniform(target_radius + organ_radius + 5.0, target_radius + organ_radius + 35.0)
        if np.sum(((np.abs(c) + organ_radius) / semi) ** 2) <= 1.0:
            break
    centres = [ph.uniform_edges(-0.5 * l, 0.5 * l, n) for l, n in zip(wl.lxyz, wl.nxyz)]
    x, y, z = [0.5 * (e[1:] + e[:-1]).astype(np.float64) for e in centres]
    r2t = (z[:, None, None] ** 2 + y[None, :, None] ** 2 + x[None, None, :] ** 2)
    r2o = ((z[:, None, None] - c[2]) ** 2 + (y[None, :, None] - c[1]) ** 2 + (x[None, None, :] - c[0]) ** 2)
    return (r2t <= target_radius ** 2).ravel(), (r2o <= organ_radius ** 2).ravel(), c


WORKLOADS = {"c1": c1, "c2": c2, "c3": c3}
