"""The multi-GPU path of the batched benchmark, on CPU with gloo ranks (2 and 3).

The job's chains are one seeded set (nchains per GPU); bench.rank_chains gives each rank its shard
by a greedy longest-first partition of the chains' atom counts (systems.shard_chains).  Checked:
the shards are disjoint and cover the set, the heaviest and lightest rank differ by at most the
largest chain, each rank builds exactly its chains (bitwise the chains of a one-rank build), and
the whole-job figures (bench.aggregate: units of all ranks over the slowest rank's time) equal the
sums of a one-process run over all chains.  The per-chain work here is the CPU oracle's Metropolis
run (a few moves, seeded by the chain's global index), so the counts do not depend on which rank
runs a chain.
"""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SIZES = dict(nmin=512, nmax=720)
PER_GPU = 3
MOVES = 4


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _chain_work(s, index):
    """Accepted moves of a short oracle Metropolis run of one chain (deterministic per chain)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    o = orc.Oracle(s)
    o.set_acceptance_units("physical")
    _, _, nacc = o.mc_run(MOVES, 100 + index, trace=False)
    return nacc


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        chains, mine = bench.rank_chains(rank, world, PER_GPU, **SIZES)
        acc = sum(_chain_work(c, i) for c, i in zip(chains, mine))
        atoms = sum(c.natom for c in chains)
        red = bench.Reducer(world, "cpu")
        # rank r's chains ran in 10 (r + 1) ms
        agg = bench.aggregate(red, float(acc), float(MOVES * len(chains)), float(atoms), 10.0 * (rank + 1))
        out[rank] = dict(mine=list(mine), atoms=atoms, agg=agg, first_x=[float(c.x[0]) for c in chains])
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_ranks_shard_one_chain_set_and_aggregate(world):
    sys.path.insert(0, ROOT)
    import bench
    from mc_cpp_gb300 import systems
    specs = bench.job_specs(PER_GPU, world, **SIZES)
    whole = systems.water_chains(nchains=PER_GPU * world, seed=bench.CHAIN_SEED, **SIZES)
    want_acc = sum(_chain_work(c, i) for i, c in enumerate(whole))
    # spawned, not forked: this process has started OpenMP thread pools
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    shards = [res[r]["mine"] for r in range(world)]
    flat = sorted(i for sh in shards for i in sh)
    assert flat == list(range(len(specs)))                       # disjoint and complete
    loads = [res[r]["atoms"] for r in range(world)]
    assert max(loads) - min(loads) <= max(3 * n for n, _, _ in specs)
    for r in range(world):                                        # each rank built exactly its chains
        assert res[r]["first_x"] == [float(whole[i].x[0]) for i in shards[r]]
    aggs = [res[r]["agg"] for r in range(world)]
    assert all(a == aggs[0] for a in aggs)                        # every rank sees the job-wide figures
    a = aggs[0]
    assert a["ms_max"] == 10.0 * world                           # the slowest rank's time
    assert a["accepted_per_s"] == pytest.approx(want_acc / (a["ms_max"] * 1e-3))
    assert a["trials_per_s"] == pytest.approx(MOVES * len(specs) / (a["ms_max"] * 1e-3))
    assert a["pairs_per_s"] == pytest.approx(sum(c.natom for c in whole) / (a["ms_max"] * 1e-3))


def test_shard_chains_balances_and_covers():
    sys.path.insert(0, ROOT)
    from mc_cpp_gb300 import systems
    rng = np.random.default_rng(0)
    w = rng.integers(1536, 24576, 256)
    for world in (1, 2, 3, 8):
        parts = systems.shard_chains(w, world)
        assert sorted(i for p in parts for i in p) == list(range(len(w)))
        loads = [int(w[p].sum()) for p in parts]
        assert max(loads) - min(loads) <= w.max()
    assert systems.shard_chains([5, 3, 3, 2, 2, 1], 2) == [[0, 3, 5], [1, 2, 4]]
    with pytest.raises(ValueError):
        systems.shard_chains([1, 2], 0)
