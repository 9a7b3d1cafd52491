"""The multi-GPU path of bench.py on two CPU ranks (gloo): structures are
sharded by rank with no data-path collective, and the only collective - the
max-over-ranks reduction of the step time - gives every rank the slowest
rank's time.  Runs without a GPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    import numpy as np
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "calypso-gap_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dev = torch.device("cpu")
        seeds = bench.shard_seeds(rank, 3)
        structs, (off, sp, lat, pos) = bench.workload(rank, 3)
        # every rank's cells are its own seeds' cells
        import gapgb.synth as S
        assert np.array_equal(pos[:512], S.alloy512(seed=seeds[0])[1])
        gathered = [None] * world
        dist.all_gather_object(gathered, seeds)
        # slowest rank's time for every rank
        t = bench.max_over_ranks(10.0 + rank, world, dev)
        out[rank] = (gathered, t, int(off[-1]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    seeds0, t0, n0 = res[0]
    seeds1, t1, n1 = res[1]
    assert seeds0 == seeds1  # the gathered lists agree
    all_seeds = [s for r in seeds0 for s in r]
    assert len(set(all_seeds)) == len(all_seeds) == world * 3  # disjoint shards
    assert t0 == t1 == 11.0  # max over ranks
    assert n0 == n1 == 3 * 512
