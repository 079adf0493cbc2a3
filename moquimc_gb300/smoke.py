"""Smoke check: one small transport on cuda:0 through the C ABI, checked against the oracle.

Transports 200 histories of the phantom example (debug physics) on the GPU and with the C
restatement on the same Philox streams, and walks 64 golden rays; raises on any mismatch.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run() -> None:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mqo  # the oracle: checker only

    from . import capi, phantom as ph, workloads

    wl = workloads.c1(histories=200)
    n = 200
    v = wl.vertices(n, 1)
    with capi.Context(0) as c:
        c.set_physics(True)
        cid = c.add_child(*wl.edges())
        c.set_hu(cid, wl.hu)
        sid = c.add_scorer(cid, capi.EDEP)
        c.set_vertices(v)
        c.transport(0, n, 2026)
        gpu = c.tally(sid)
        st = c.stats()
        g = np.load(os.path.join(ROOT, "tests", "golden", "raywalk.npz"))
        b, nn = g["phantom_bounds"], g["phantom_n"]
        edges = [ph.uniform_edges(float(b[2 * a]), float(b[2 * a + 1]), int(nn[a])) for a in range(3)]
        rid = c.add_child(*edges)
        rays = g["phantom_rays"][:64]
        off, cnb, dist, _ = c.trace_rays(rid, rays, int(g["phantom_max_steps"]))
    k = int(off[-1])
    if not (np.array_equal(off, g["phantom_offsets"][:65]) and np.array_equal(cnb.astype(np.uint32), g["phantom_cnb"][:k])
            and np.array_equal(dist.view(np.uint32), g["phantom_dist_bits"][:k])):
        raise AssertionError("smoke: voxel walk differs from the reference")
    rho = np.full(int(np.prod(wl.nxyz)), mqo.hu_to_density(0), np.float32)
    ora, _, ost = mqo.transport(mqo.Grid(*wl.edges(), rho), v, 0, n, 2026, True, scorer=1)
    if st["histories"] != n or abs(gpu.sum() - ora.sum()) > 1e-3 * ora.sum():
        raise AssertionError(f"smoke: GPU energy {gpu.sum()} vs oracle {ora.sum()} ({st}, {ost})")
    print(f"smoke ok: {n} histories, {st['steps']} steps, energy GPU {gpu.sum():.6g} MeV vs oracle {ora.sum():.6g} MeV")


if __name__ == "__main__":
    run()
