"""The multi-GPU replica path on the CPU: two gloo ranks each transport their own histories (the
C restatement stands in for the GPU), then the FP64 tallies are summed and the step time is the
maximum over ranks -- the exchange bench.py performs under torchrun."""
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_setup():
    from moquimc_gb300 import phantom as ph

    nxyz, lxyz, pxyz = (24, 24, 60), (24.0, 24.0, 60.0), (0.0, 0.0, -30.0)
    edges = ph.phantom_box_edges(lxyz, pxyz, nxyz)
    return edges, nxyz


def _run_rank(rank, world_size, port, out_dir):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world_size),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import mqo
    from moquimc_gb300 import phantom as ph
    from moquimc_gb300 import replicas

    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    ws, rk, _ = replicas.world()
    edges, nxyz = _replica_setup()
    grid = mqo.Grid(*edges, np.full(int(np.prod(nxyz)), mqo.hu_to_density(0), np.float32))
    vseed, tseed = replicas.replica_seeds(rk)
    v = ph.gaussian_spot_vertices(40, np.random.default_rng(vseed), 60.0, (0.0, 0.0, 0.5), (2.0, 2.0))
    tally, _, st = mqo.transport(grid, v, 0, len(v), tseed, False)
    total = replicas.sum_tallies(tally).numpy()
    tmax = replicas.max_over_ranks(1.0 + rk)
    np.save(os.path.join(out_dir, f"tally{rk}.npy"), tally)
    if rk == 0:
        np.save(os.path.join(out_dir, "total.npy"), total)
        np.save(os.path.join(out_dir, "tmax.npy"), np.array([tmax, ws]))
    dist.destroy_process_group()


def test_two_gloo_replicas_sum_their_tallies(tmp_path, oracle):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from moquimc_gb300 import replicas

    port = _free_port()
    mp.start_processes(_run_rank, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    t0, t1 = np.load(tmp_path / "tally0.npy"), np.load(tmp_path / "tally1.npy")
    total = np.load(tmp_path / "total.npy")
    assert t0.sum() > 0 and t1.sum() > 0 and not np.array_equal(t0, t1)   # independent replicas
    np.testing.assert_array_equal(total, t0 + t1)
    tmax, ws = np.load(tmp_path / "tmax.npy")
    assert tmax == 2.0 and ws == 2
    # rank-local seeds are distinct and the strong-scaling split covers every history once
    assert len({replicas.replica_seeds(r) for r in range(8)}) == 8
    cover = [replicas.history_range(1003, r, 4) for r in range(4)]
    assert cover[0][0] == 0 and cover[-1][1] == 1003 and all(a[1] == b[0] for a, b in zip(cover, cover[1:]))
    assert torch is not None
