"""The multi-GPU path of the batched benchmark, on CPU with two gloo ranks: every rank builds its
own chains (different seeds, no data exchanged) and the whole-job rates are the sum of all ranks'
units over the slowest rank's time."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        chains = bench.make_chains(rank, 3, nmin=512, nmax=700)
        red = bench.Reducer(world, "cpu")
        # rank r pretends to have accepted 100 (r + 1) moves of 1000 (r + 1) trials in 10 (r + 1) ms
        agg = bench.aggregate(red, 100.0 * (rank + 1), 1000.0 * (rank + 1), 5000.0 * (rank + 1), 10.0 * (rank + 1))
        out[rank] = (agg, [c.natom for c in chains], float(chains[0].x[0]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_chains_and_aggregate():
    world = 2
    # spawned, not forked: earlier tests in this process may have started thread pools (OpenMP)
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    a0, n0, x0 = res[0]
    a1, n1, x1 = res[1]
    assert a0 == a1                                   # every rank sees the same job-wide figures
    assert a0["ms_max"] == 20.0                      # the slowest rank's time
    assert a0["accepted_per_s"] == pytest.approx((100 + 200) / 0.020)
    assert a0["trials_per_s"] == pytest.approx((1000 + 2000) / 0.020)
    assert a0["pairs_per_s"] == pytest.approx((5000 + 10000) / 0.020)
    assert (n0, x0) != (n1, x1)                      # each rank built its own chains
