"""mqi_transport_noalloc: the allocation-free transport for callers that cannot call cudaMalloc
once running (memory owned by a pre-sized pool or another framework's allocator, plug-in hosts
that forbid allocation after start-up).  Its queues live in a static device array inside the
library; every other buffer is the caller's.

The test allocates the caller's buffers itself (with torch), calls the entry point through the C
ABI twice in a row, and checks each result against the context-based mqi_transport on the same
inputs and seed: the same kernels and random streams, so the tallies agree to FP64 summation order.
This file is collected last so that a run stopping at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest

from moquimc_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_transport_matches_context_transport_on_two_calls(built_lib):
    import torch

    wl = workloads.c2()
    n = 150_000                      # three 65536-primary generations of the static queues
    verts = wl.vertices(n, 77)
    xe, ye, ze = wl.edges()
    nx, ny, nz = wl.nxyz
    seeds = (0x5EED01, 0x5EED02)

    # reference results: the existing context-based entry point
    ref = []
    with capi.Context(0) as c:
        c.set_physics(wl.physics_debug)
        cid = c.add_child(xe, ye, ze)
        c.set_hu(cid, wl.hu)
        sid = c.add_scorer(cid, capi.DOSE_W)
        rho = c.hu_to_density(wl.hu.reshape(-1))
        c.set_vertices(verts)
        for s in seeds:
            c.reset()
            c.transport(0, n, s)
            ref.append(c.tally(sid))

    # the caller's device buffers (the entry point allocates nothing)
    dev = torch.device("cuda", 0)
    d_xe = torch.from_numpy(xe).to(dev)
    d_ye = torch.from_numpy(ye).to(dev)
    d_ze = torch.from_numpy(ze).to(dev)
    d_rho = torch.from_numpy(rho).to(dev)
    d_v = torch.from_numpy(verts.view(np.uint8).copy()).to(dev)
    stream = torch.cuda.current_stream(dev)
    for s, expect in zip(seeds, ref):
        d_tally = torch.zeros(nx * ny * nz, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = built_lib.mqi_transport_noalloc(nx, ny, nz, _ptr(d_xe), _ptr(d_ye), _ptr(d_ze), _ptr(d_rho), _ptr(d_v), n,
                                             capi.DOSE_W, int(wl.physics_debug), s, _ptr(d_tally),
                                             ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, built_lib.mqi_last_error(None)
        got = d_tally.cpu().numpy()
        assert got.sum() > 0
        np.testing.assert_allclose(got, expect, rtol=1e-9, atol=1e-300)


_SCORERS = {"edep": capi.EDEP, "dose_w": capi.DOSE_W, "dose_w2": capi.DOSE_W2, "dose_m": capi.DOSE_M}


@pytest.mark.parametrize("physics_debug", [0, 1])
@pytest.mark.parametrize("scorer", sorted(_SCORERS))
def test_noalloc_every_scorer_and_physics_build(built_lib, scorer, physics_debug):
    """Every scorer the entry point accepts (each selects its own kernel instance: EDEP and DOSE_W
    the single-scorer one, DOSE_W2 the generic one, DOSE_M the one with the FP64 callbacks), with
    release and debug physics, on a history count that is not a multiple of the 65536-primary
    generation; two calls in a row, each against the context transport."""
    import torch

    wl = workloads.c2()
    n = 65_536 + 4_465
    stype = _SCORERS[scorer]
    verts = wl.vertices(n, 91)
    xe, ye, ze = wl.edges()
    nx, ny, nz = wl.nxyz
    seeds = (0xA11C0C, 0xA11C0D)
    ref = []
    with capi.Context(0) as c:
        c.set_physics(physics_debug)
        cid = c.add_child(xe, ye, ze)
        c.set_hu(cid, wl.hu)
        sid = c.add_scorer(cid, stype)
        rho = c.hu_to_density(wl.hu.reshape(-1))
        c.set_vertices(verts)
        for s in seeds:
            c.reset()
            c.transport(0, n, s)
            ref.append(c.tally(sid))
    dev = torch.device("cuda", 0)
    d_xe, d_ye, d_ze, d_rho = (torch.from_numpy(a).to(dev) for a in (xe, ye, ze, rho))
    d_v = torch.from_numpy(verts.view(np.uint8).copy()).to(dev)
    stream = torch.cuda.current_stream(dev)
    d_tally = torch.zeros(nx * ny * nz, dtype=torch.float64, device=dev)
    for s, expect in zip(seeds, ref):
        d_tally.zero_()
        torch.cuda.synchronize()
        rc = built_lib.mqi_transport_noalloc(nx, ny, nz, _ptr(d_xe), _ptr(d_ye), _ptr(d_ze), _ptr(d_rho), _ptr(d_v), n,
                                             stype, physics_debug, s, _ptr(d_tally),
                                             ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, built_lib.mqi_last_error(None)
        got = d_tally.cpu().numpy()
        assert got.sum() > 0
        np.testing.assert_allclose(got, expect, rtol=1e-9, atol=1e-300)


def test_noalloc_rejects_sizes_beyond_its_limit(built_lib):
    rc = built_lib.mqi_transport_noalloc(8, 8, 8, ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1),
                                         ctypes.c_void_p(1), ctypes.c_void_p(1), (1 << 24) + 1, capi.DOSE_W, 0, 1,
                                         ctypes.c_void_p(1), None)
    assert rc == -1
    assert b"16777216" in built_lib.mqi_last_error(None)
