"""Phantom and beam set-up helpers that mirror moqui's phantom_env on the host side.

The voxel edges are computed with the same FP32 arithmetic as moqui's grid3d uniform-edge
constructor (moqui/base/mqi_grid3d.hpp: dx = (max - min) / n; edge_i = min + i * dx) from the box
corners phantom_env::setup_world derives from --lxyz/--pxyz (mqi_phantom_env.hpp:256-264), so a
grid built here holds bit-identical edges.
"""
from __future__ import annotations

import numpy as np

from .capi import VERTEX_DTYPE

f32 = np.float32


def uniform_edges(lo: float, hi: float, n: int) -> np.ndarray:
    """grid3d(xe_min, xe_max, n+1, ...) edge array in FP32."""
    lo, hi = f32(lo), f32(hi)
    dx = f32(hi - lo) / f32(n)
    i = np.arange(n + 1, dtype=np.float32)
    return (lo + (i * dx).astype(np.float32)).astype(np.float32)


def phantom_box_edges(lxyz, pxyz, nxyz):
    """Edges of phantom_env's child grid: corners pos -/+ 0.5 * l, computed in double then stored
    as float (x[0] = pos.x - 0.5 * lxyz.x in mqi_phantom_env.hpp:256-261)."""
    out = []
    for l, p, n in zip(lxyz, pxyz, nxyz):
        l32, p32 = float(f32(l)), float(f32(p))
        lo = float(f32(p32 - 0.5 * l32))
        hi = float(f32(p32 + 0.5 * l32))
        out.append(uniform_edges(lo, hi, int(n)))
    return out


def uniform_spot_vertices(n: int, rng: np.random.Generator, energy: float, position=(0.0, 0.0, 0.5),
                          size=(30.0, 30.0)) -> np.ndarray:
    """phantom_env's beam (mqi_phantom_env.hpp:204-232): phsp_6d_uniform with mean
    (position, dir 0,0,-1) and half-widths `size` on x/y (distributions/mqi_phsp6d_uniform.hpp:66-85),
    constant energy (const_1d)."""
    v = np.zeros(n, dtype=VERTEX_DTYPE)
    v["ke"] = f32(energy)
    ux = rng.uniform(-1.0, 1.0, n).astype(np.float32)
    uy = rng.uniform(-1.0, 1.0, n).astype(np.float32)
    v["pos"][:, 0] = f32(position[0]) + f32(size[0]) * ux
    v["pos"][:, 1] = f32(position[1]) + f32(size[1]) * uy
    v["pos"][:, 2] = f32(position[2])
    v["dir"][:, 2] = f32(-1.0)
    return v


def gaussian_spot_vertices(n: int, rng: np.random.Generator, energy: float, position=(0.0, 0.0, 0.5),
                           sigma=(4.0, 4.0)) -> np.ndarray:
    """phsp_6d (distributions/mqi_phsp6d.hpp:61-79) with zero divergence: Gaussian x/y of the
    given sigma, direction (0,0,-1), constant energy."""
    v = np.zeros(n, dtype=VERTEX_DTYPE)
    v["ke"] = f32(energy)
    v["pos"][:, 0] = f32(position[0]) + f32(sigma[0]) * rng.standard_normal(n).astype(np.float32)
    v["pos"][:, 1] = f32(position[1]) + f32(sigma[1]) * rng.standard_normal(n).astype(np.float32)
    v["pos"][:, 2] = f32(position[2])
    v["dir"][:, 2] = f32(-1.0)
    return v


def depth_dose(dose: np.ndarray, nxyz) -> np.ndarray:
    """Laterally integrated depth dose from a flat [nz][ny][nx] tally, ordered from the beam
    entrance (the largest z index, since the beam travels along -z) downwards."""
    nx, ny, nz = nxyz
    return dose.reshape(nz, ny, nx).sum(axis=(1, 2))[::-1].copy()


def r80(idd: np.ndarray, dz: float) -> float:
    """Distal depth (mm from the entrance surface) where the depth dose falls to 80% of its maximum,
    by linear interpolation between voxel centres."""
    i = int(np.argmax(idd))
    m = idd[i]
    tail = np.where(idd[i:] < 0.8 * m)[0]
    if len(tail) == 0:
        return float("nan")
    j = i + int(tail[0])
    frac = (idd[j - 1] - 0.8 * m) / (idd[j - 1] - idd[j])
    return float(((j - 1) + 0.5 + frac) * dz)


def column_crop(dose: np.ndarray, lxyz, nxyz, x: float, y: float, half: int = 24, bins=(7, 7, 4)) -> np.ndarray:
    """The (2 half + 1)^2-voxel column around the beam axis (x, y) of a grid centred at the origin,
    summed in bins (bx, by, bz): shape (nz / bz, (2 half + 1) / by, (2 half + 1) / bx)."""
    nx, ny, nz = nxyz
    d = dose.reshape(nz, ny, nx)
    ix = int((x + 0.5 * lxyz[0]) / (lxyz[0] / nx))
    iy = int((y + 0.5 * lxyz[1]) / (lxyz[1] / ny))
    w = 2 * half + 1
    c = d[:, iy - half:iy + half + 1, ix - half:ix + half + 1]
    bx, by, bz = bins
    return c.reshape(nz // bz, bz, w // by, by, w // bx, bx).sum(axis=(1, 3, 5))

