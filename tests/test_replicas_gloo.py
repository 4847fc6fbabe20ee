"""Replica path on CPU: two gloo ranks exercise the host logic that bench.py,
the warm-start data generation and the difference-quotient gradient run with
one process per GPU — the max-over-ranks step time, the barrier, the contiguous
sharding of independent units (site tensors, gradient elements) and the gather
of every rank's share in rank order."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    import __graft_entry__ as ge

    tn = ge.load_package()
    import importlib

    wl = importlib.import_module(tn.__name__ + ".learned")
    dist, r, w = bench.dist_init(world, backend="gloo")
    try:
        bench.barrier(dist)
        t = bench.max_over_ranks(dist, 1.0 + 2.5 * r)
        mine = list(wl.shard_range(11, r, w))
        allv = wl.gather_shards([10 * i for i in mine], dist)
        K = np.arange(30, dtype=np.float64).reshape(2, 3, 5) / 7.0
        g = tn.num_grad(lambda x: float(np.sum(x ** 3)), K, 1e-4, dist=dist)
        q.put((r, t, mine, allv, g))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_shard_and_gather():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[1] for o in out] == [3.5, 3.5]  # every rank sees the slowest rank's time
    assert out[0][2] + out[1][2] == list(range(11))  # contiguous, disjoint, complete
    assert out[0][3] == out[1][3] == [10 * i for i in range(11)]
    K = np.arange(30, dtype=np.float64).reshape(2, 3, 5) / 7.0
    for o in out:  # each rank differentiated half of the elements; both hold all of them
        assert np.allclose(o[4], 3 * K ** 2, rtol=1e-8, atol=1e-8)


def test_shard_range_covers_every_unit_once():
    sys.path.insert(0, str(ROOT))
    import importlib

    import __graft_entry__ as ge

    wl = importlib.import_module(ge.load_package().__name__ + ".learned")
    for n in (0, 1, 7, 500):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in wl.shard_range(n, r, world)]
            assert got == list(range(n))
