"""Synthetic workloads of the benchmark configurations (seeded; no patient data exists).

* ``c1``: moqui's phantom example -- a 100x100x350 mm water box (HU 0) of 200x200x350 voxels,
  one 200 MeV spot with a uniform +-30 mm square profile, 1e5 histories, debug physics (the
  example is built with -D__PHYSICS_DEBUG__).
* ``c2``: a 256^3 phantom of 1 mm voxels centred at (0, 0, -128): water (HU 0) with a 30 mm lung
  slab (HU -700) and a 15 mm bone slab (HU 1200) at depths drawn from numpy's default_rng(2) in
  40-180 mm, full lateral extent; one 150 MeV Gaussian spot (sigma 4 mm), 1e6 histories.
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


WORKLOADS = {"c1": c1, "c2": c2}
