"""Multi-GPU sharding of a packed batch of structures (one process per GPU).

Structures are independent, so a batch is split by whole structures with no
collective on the data path; the only exchange is the gather of every
structure's energy, forces and stress to rank 0 at the end.

- ``shard_structures``: greedy balance by atom count (largest structure
  first, onto the rank with the fewest atoms so far).  For the population's
  8-256-atom cells this keeps the ranks' atom counts within one structure of
  each other: the rank that ends up largest received its last structure
  while it was the smallest.
- ``local_batch``: the packed (atom_off, species, lat, pos) of one rank's
  structures.
- ``gather_results``: all ranks' (E, F, stress) reassembled on rank 0 in the
  original structure order, through one all_gather of padded float64
  buffers (NCCL between GPUs, gloo on the host); every rank derives the
  layout from the same deterministic shard lists, so no sizes are exchanged.
"""
import numpy as np


def shard_structures(atom_off, world):
    """Structure indices of each rank (ascending within a rank)."""
    off = np.asarray(atom_off, np.int64)
    counts = np.diff(off)
    order = np.argsort(-counts, kind="stable")
    load = np.zeros(world, np.int64)
    owner = np.empty(len(counts), np.int64)
    for s in order:
        r = int(np.argmin(load))  # the first rank among equals
        owner[s] = r
        load[r] += counts[s]
    return [np.flatnonzero(owner == r) for r in range(world)]


def local_batch(atom_off, species, lat, pos, idx):
    """Packed batch of the structures `idx` (in that order)."""
    off = np.asarray(atom_off, np.int64)
    idx = np.asarray(idx, np.int64)
    counts = off[idx + 1] - off[idx]
    loff = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    rows = np.concatenate([np.arange(off[s], off[s + 1]) for s in idx]) if len(idx) else \
        np.zeros(0, np.int64)
    lat = np.asarray(lat).reshape(-1, 3, 3)
    return (loff, np.asarray(species)[rows].astype(np.int32), lat[idx].copy(),
            np.asarray(pos).reshape(-1, 3)[rows].copy())


def _layout(atom_off, shard):
    off = np.asarray(atom_off, np.int64)
    n_atoms = int((off[shard + 1] - off[shard]).sum())
    return len(shard), n_atoms, 7 * len(shard) + 3 * n_atoms


def gather_results(E, F, S, atom_off, shards, rank, device=None):
    """(E[S], F[N, 3], stress[S, 6]) of the whole batch on rank 0 (None on
    the other ranks).  E, F, S are this rank's results for its shard, in the
    order of shards[rank]; torch tensors or numpy arrays."""
    import torch
    import torch.distributed as dist
    world = len(shards)
    sizes = [_layout(atom_off, sh)[2] for sh in shards]
    width = max(max(sizes), 1)
    dev = device if device is not None else torch.device("cpu")

    def t(a):
        return torch.as_tensor(a, dtype=torch.float64).reshape(-1).to(dev)

    mine = torch.zeros(width, dtype=torch.float64, device=dev)
    flat = torch.cat([t(E), t(S), t(F)])
    mine[:flat.numel()] = flat
    bufs = [torch.zeros(width, dtype=torch.float64, device=dev) for _ in range(world)]
    dist.all_gather(bufs, mine)
    if rank != 0:
        return None
    off = np.asarray(atom_off, np.int64)
    ns = len(off) - 1
    E_all = np.zeros(ns)
    S_all = np.zeros((ns, 6))
    F_all = np.zeros((int(off[-1]), 3))
    for r, sh in enumerate(shards):
        b = bufs[r].cpu().numpy()
        k, na, _ = _layout(atom_off, sh)
        E_all[sh] = b[:k]
        S_all[sh] = b[k:7 * k].reshape(k, 6)
        Fr = b[7 * k:7 * k + 3 * na].reshape(na, 3)
        a = 0
        for s in sh:
            n = int(off[s + 1] - off[s])
            F_all[off[s]:off[s + 1]] = Fr[a:a + n]
            a += n
    return E_all, F_all, S_all
