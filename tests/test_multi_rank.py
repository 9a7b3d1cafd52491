"""The multi-GPU path on two CPU ranks (gloo), without a GPU: structures are
sharded by rank with no data-path collective; the max-over-ranks reduction
of the step time gives every rank the slowest rank's time; and a ragged
batch sharded by atom count (gapgb.shard) is evaluated rank by rank (here by
the CPU oracle) and gathered to rank 0 equal to a single-rank evaluation."""
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


def _ragged_batch():
    import numpy as np
    import gapgb.synth as S
    rng = np.random.default_rng(31)
    return [S.random_structure(rng, n, species_pool=(3, 8, 14, 26))
            for n in (9, 40, 17, 33, 12, 25, 8, 21, 30, 14)]


def _gather_main(rank, world, port, model_path, out):
    import sys
    import numpy as np
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "calypso-gap_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import gapgb.synth as S
    from gapgb import shard
    from oracle import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        structs = _ragged_batch()
        off, sp, lat, pos = S.pack(structs)
        shards = shard.shard_structures(off, world)
        loff, lsp, llat, lpos = shard.local_batch(off, sp, lat, pos, shards[rank])
        om = oracle.Model(model_path)
        E, F, St = [], [], []
        for q in range(len(loff) - 1):
            a, b = loff[q], loff[q + 1]
            e, f, s_, _ = oracle.gap_calc(om, lsp[a:b], llat[q], lpos[a:b], 6.0, True)
            E.append(e), F.append(f), St.append(s_)
        res = shard.gather_results(np.array(E), np.concatenate(F), np.array(St), off, shards,
                                   rank)
        out[rank] = (res, [int(np.diff(off)[sh].sum()) for sh in shards],
                     [sh.tolist() for sh in shards], int(np.diff(off).max()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_atom_balanced_shards_gather_to_rank0(oracle_mod, tmp_path):
    import numpy as np
    import torch.multiprocessing as mp
    import gapgb.synth as S
    from helpers import synth_model_file
    structs = _ragged_batch()
    path = synth_model_file(str(tmp_path / "gap_parameters"), oracle_mod, structs, M=60,
                            theta_scale=2.0, coeff_std=0.5, seed=3, zeta=False)
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_gather_main, args=(world, port, path, out), nprocs=world, join=True)
        res = dict(out)
    (E, F, St), atoms, shards, biggest = res[0]
    assert res[1][0] is None  # only rank 0 receives the results
    # every structure once, and the ranks' atom counts within one structure
    assert sorted(shards[0] + shards[1]) == list(range(len(structs)))
    assert abs(atoms[0] - atoms[1]) <= biggest
    # gathered results equal a single-rank evaluation, in the original order
    om = oracle_mod.Model(path)
    off, sp, lat, pos = S.pack(structs)
    for s, (l, p, z) in enumerate(structs):
        e, f, s_, _ = oracle_mod.gap_calc(om, z, l, p, 6.0, True)
        assert E[s] == e
        assert np.array_equal(F[off[s]:off[s + 1]], f)
        assert np.array_equal(St[s], s_)


def test_shard_structures_balances_atoms():
    import numpy as np
    from gapgb import shard
    rng = np.random.default_rng(5)
    counts = rng.integers(8, 257, 8192)
    off = np.concatenate([[0], np.cumsum(counts)])
    for world in (2, 4, 8):
        shards = shard.shard_structures(off, world)
        loads = [int(counts[sh].sum()) for sh in shards]
        assert sorted(np.concatenate(shards).tolist()) == list(range(len(counts)))
        assert max(loads) - min(loads) <= counts.max()
