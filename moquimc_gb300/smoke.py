"""Smoke check: small transports on cuda:0 through the C ABI, checked against the oracle.

1. 64 golden rays walked through the phantom grid: bit-exact against the reference's walk.
2. The phantom example (debug physics) on 10 x 10 coarser lateral voxels, 200 histories one at a
   time on the GPU and in the C restatement on the same Philox streams: a history deposits the
   same energy (to 1e-4) unless an FP32 rounding difference flips one discrete decision along it,
   so at least 90% of them must agree and the totals within 2%.
3. The phantom example at full resolution, 200 histories in one launch: every history
   transported, no bounded device loop gave up, and the energy within 2% of the oracle's (the
   rotation's FP32 rounding differs from the reference's formula, so more histories diverge
   here and only the total is compared).
Raises AssertionError on any mismatch.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _context(capi, wl):
    c = capi.Context(0)
    c.set_physics(True)
    cid = c.add_child(*wl.edges())
    c.set_hu(cid, wl.hu)
    return c, cid, c.add_scorer(cid, capi.EDEP)


def run() -> None:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mqo  # the oracle: checker only

    from . import capi, phantom as ph, workloads

    n, seed = 200, 2026
    # 1. voxel walk
    g = np.load(os.path.join(ROOT, "tests", "golden", "raywalk.npz"))
    b, nn = g["phantom_bounds"], g["phantom_n"]
    edges = [ph.uniform_edges(float(b[2 * a]), float(b[2 * a + 1]), int(nn[a])) for a in range(3)]
    with capi.Context(0) as c:
        rid = c.add_child(*edges)
        off, cnb, dist, _ = c.trace_rays(rid, g["phantom_rays"][:64], int(g["phantom_max_steps"]))
    k = int(off[-1])
    if not (np.array_equal(off, g["phantom_offsets"][:65]) and np.array_equal(cnb.astype(np.uint32), g["phantom_cnb"][:k])
            and np.array_equal(dist.view(np.uint32), g["phantom_dist_bits"][:k])):
        raise AssertionError("smoke: voxel walk differs from the reference")

    # 2. history by history on coarse lateral voxels
    wl = workloads.c1(histories=n)
    nx, ny, nz = wl.nxyz
    wl.hu = np.ascontiguousarray(wl.hu[:, ::10, ::10])
    wl.nxyz = (nx // 10, ny // 10, nz)
    v = wl.vertices(n, 1)
    e_gpu = np.zeros(n)
    c, _, sid = _context(capi, wl)
    with c:
        c.set_vertices(v)
        for h in range(n):
            c.reset()
            c.transport(h, h + 1, seed)
            e_gpu[h] = c.tally(sid).sum()
    rho = np.full(int(np.prod(wl.nxyz)), mqo.hu_to_density(0), np.float32)
    _, e_ora, _ = mqo.transport(mqo.Grid(*wl.edges(), rho), v, 0, n, seed, True, scorer=1, per_history=True)
    same = float(np.mean(np.abs(e_gpu - e_ora) <= 1e-4 * np.maximum(e_ora, 1e-9)))
    if same < 0.9 or abs(e_gpu.sum() - e_ora.sum()) > 0.02 * e_ora.sum():
        raise AssertionError(f"smoke: {same:.3f} of the histories agree with the oracle; energy GPU "
                             f"{e_gpu.sum()} vs oracle {e_ora.sum()} MeV")

    # 3. one launch at full resolution
    wl = workloads.c1(histories=n)
    v = wl.vertices(n, 1)
    c, _, sid = _context(capi, wl)
    with c:
        c.set_vertices(v)
        c.transport(0, n, seed)
        gpu = c.tally(sid)
        st = c.stats()
    rho = np.full(int(np.prod(wl.nxyz)), mqo.hu_to_density(0), np.float32)
    ora, _, _ = mqo.transport(mqo.Grid(*wl.edges(), rho), v, 0, n, seed, True, scorer=1)
    if st["histories"] != n or st["device_errors"] != 0 or abs(gpu.sum() - ora.sum()) > 0.02 * ora.sum():
        raise AssertionError(f"smoke: GPU energy {gpu.sum()} vs oracle {ora.sum()} MeV ({st})")
    print(f"smoke ok: {same:.3f} of {n} histories identical to the oracle on coarse voxels; full grid "
          f"{st['steps']} steps, energy GPU {gpu.sum():.6g} MeV vs oracle {ora.sum():.6g} MeV")


if __name__ == "__main__":
    run()
