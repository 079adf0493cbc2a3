"""Beamline children: range shifters and voxelised apertures placed in the world before the patient.

moqui's tps_env builds one child per beamline device and puts them before the patient
(moqui/base/environments/mqi_tps_env.hpp:735-758): a range shifter is a single-voxel box filled
with the shifter's density (create_rangeshifter, :1605-1650); an aperture is a 1 mm voxel grid
whose columns inside the opening hold 1e-8 g/mm^3 (vacuum for the transport) and elsewhere 100
g/mm^3, which stops every track that enters it (create_voxelized_aperture, :1652-1737).  Both carry
the beam's rotation and translation.  The transport walks the children in order for every track
(mqi_transport.hpp:161-239), which is what `Context.add_child` reproduces; these helpers build the
edges and densities, and `add_to` adds a child to a context.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

APERTURE_OPEN = np.float32(1.0e-8)     # g/mm^3: below the 1e-7 vacuum threshold
APERTURE_BLOCK = np.float32(100.0)     # g/mm^3: above the 99.9 stop threshold


def rotation_xyz(ax: float, ay: float, az: float) -> np.ndarray:
    """mat3x3(a, b, c) (moqui/base/mqi_matrix.hpp:69-76, 213-270): the identity rotated about x,
    then y, then z by the given angles in radians (a zero angle is skipped).  Row-major 3x3."""
    xx, xy, xz, yx, yy, yz, zx, zy, zz = 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0
    f = np.float32
    ax, ay, az = (float(f(a)) for a in (ax, ay, az))   # the FP32 angle, as mat3x3<float> holds it
    if ax != 0:
        c, s = f(math.cos(ax)), f(math.sin(ax))
        x1, y1, z1 = f(yx), f(yy), f(yz)
        yx, yy, yz = c * x1 - s * f(zx), c * y1 - s * f(zy), c * z1 - s * f(zz)
        zx, zy, zz = s * x1 + c * f(zx), s * y1 + c * f(zy), s * z1 + c * f(zz)
    if ay != 0:
        c, s = f(math.cos(ay)), f(math.sin(ay))
        x1, y1, z1 = f(zx), f(zy), f(zz)
        zx, zy, zz = c * x1 - s * f(xx), c * y1 - s * f(xy), c * z1 - s * f(xz)
        xx, xy, xz = s * x1 + c * f(xx), s * y1 + c * f(xy), s * z1 + c * f(xz)
    if az != 0:
        c, s = f(math.cos(az)), f(math.sin(az))
        x1, y1, z1 = f(xx), f(xy), f(xz)
        xx, xy, xz = c * x1 - s * f(yx), c * y1 - s * f(yy), c * z1 - s * f(yz)
        yx, yy, yz = s * x1 + c * f(yx), s * y1 + c * f(yy), s * z1 + c * f(yz)
    return np.array([xx, xy, xz, yx, yy, yz, zx, zy, zz], np.float32)


@dataclass
class BeamlineChild:
    """A child grid: edges (mm, child frame), densities (g/mm^3, x fastest), rotation
    (child -> world, row-major) and translation (mm)."""
    xe: np.ndarray
    ye: np.ndarray
    ze: np.ndarray
    rho: np.ndarray
    rot: Optional[np.ndarray] = None
    translation: Optional[np.ndarray] = None
    kind: str = ""
    meta: dict = field(default_factory=dict)

    def add_to(self, ctx) -> int:
        """Add this child to a capi.Context (after any children already added) with its densities."""
        cid = ctx.add_child(self.xe, self.ye, self.ze, rot_fwd=self.rot, translation=self.translation)
        ctx.set_density(cid, self.rho)
        return cid


def _uniform(lo: float, hi: float, n: int) -> np.ndarray:
    """grid3d's edges from (min, max, n+1 nodes) in FP32 (mqi_grid3d.hpp:217-251)."""
    lo, hi = np.float32(lo), np.float32(hi)
    d = (hi - lo) / np.float32(n)
    return (lo + np.arange(n + 1, dtype=np.float32) * d).astype(np.float32)


def range_shifter(lo: Sequence[float], hi: Sequence[float], density_g_cm3: float, rot=None,
                  translation=None) -> BeamlineChild:
    """create_rangeshifter (mqi_tps_env.hpp:1605-1650): one voxel spanning the box [lo, hi] of the
    child frame, filled with density_g_cm3 x 1e-3 g/mm^3."""
    xe, ye, ze = (_uniform(lo[a], hi[a], 1) for a in range(3))
    # fill_data(rangeshifter_density * 1e-3): the FP32 density times a double constant
    rho = np.array([np.float32(float(np.float32(density_g_cm3)) * 1e-3)], np.float32)
    return BeamlineChild(xe, ye, ze, rho, None if rot is None else np.asarray(rot, np.float32),
                         None if translation is None else np.asarray(translation, np.float32), "rangeshifter",
                         {"density_g_cm3": density_g_cm3})


def _inside_polygon(px: float, py: float, poly: np.ndarray) -> bool:
    """Crossing-number test of tps_env::sol1_1 (mqi_tps_env.hpp:1753-1770), in FP32."""
    f = np.float32
    c = False
    n = len(poly)
    j = n - 1
    for i in range(n):
        x0, y0 = f(poly[i, 0]), f(poly[i, 1])
        x1, y1 = f(poly[j, 0]), f(poly[j, 1])
        if ((y0 <= py < y1) or (y1 <= py < y0)) and (px < (x1 - x0) * (py - y0) / (y1 - y0) + x0):
            c = not c
        j = i
    return c


def voxelized_aperture(center: Sequence[float], volume: Sequence[float], openings: Sequence[np.ndarray],
                       rot=None, translation=None, voxel: float = 1.0) -> BeamlineChild:
    """create_voxelized_aperture (mqi_tps_env.hpp:1652-1737): voxels of `voxel` mm over the box of
    size `volume` centred at `center` (child frame), ceil(volume / voxel) per axis; a column whose
    voxel centre lies inside the opening is open (1e-8 g/mm^3), the rest is block (100 g/mm^3).
    The openings are polygons in the aperture plane, relative to the centre (block_data).  As in the
    reference (is_inside, :1739-1750), only the last opening decides: each one overwrites the
    result of the previous."""
    f = np.float32
    vox = f(voxel)
    dims = [int(math.ceil(float(f(volume[a]) / vox))) for a in range(3)]
    edges = []
    for a in range(3):
        lo = f(center[a]) - f(volume[a]) / f(2.0)
        edges.append((lo + np.arange(dims[a] + 1, dtype=np.float32) * vox).astype(np.float32))
    xe, ye, ze = edges
    polys = [np.asarray(p, np.float32) + np.array([f(center[0]), f(center[1])], np.float32) for p in openings]
    nx, ny, nz = dims
    col = np.empty((ny, nx), np.float32)
    for i in range(nx):
        px = f(xe[i] + vox * f(0.5))
        for j in range(ny):
            py = f(ye[j] + vox * f(0.5))
            inside = False
            for poly in polys:
                inside = _inside_polygon(px, py, poly)
            col[j, i] = APERTURE_OPEN if inside else APERTURE_BLOCK
    rho = np.broadcast_to(col, (nz, ny, nx)).astype(np.float32).reshape(-1)
    return BeamlineChild(xe, ye, ze, rho, None if rot is None else np.asarray(rot, np.float32),
                         None if translation is None else np.asarray(translation, np.float32), "aperture",
                         {"openings": len(polys)})


def children_from_devices(devices):
    """The BeamlineChild of each device: ("rangeshifter", lo, hi, density_g_cm3, angles, translation)
    or ("aperture", center, volume, openings, angles, translation); angles in radians (mat3x3)."""
    out = []
    for d in devices:
        if d[0] == "rangeshifter":
            _, lo, hi, dens, ang, tr = d
            out.append(range_shifter(lo, hi, dens, rotation_xyz(*ang), tr))
        else:
            _, center, volume, openings, ang, tr = d
            out.append(voxelized_aperture(center, volume, openings, rotation_xyz(*ang), tr))
    return out


def circle(radius: float, n: int = 64) -> np.ndarray:
    """A polygon approximating a circle of the given radius (an opening for voxelized_aperture)."""
    a = 2.0 * np.pi * np.arange(n) / n
    return np.stack([radius * np.cos(a), radius * np.sin(a)], axis=1).astype(np.float32)
