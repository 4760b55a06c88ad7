"""Multi-GPU use of the engine: independent replicas, no exchange step.

The hot path does not shard a single system (one system lives on one GPU;
a domain decomposition with a halo exchange per step is not built), so a run
on N GPUs is N independent replicas: one process per GPU, each with its own
context and engine, and only host-side scalars cross ranks (timings and
counts, reduced once at the end).  A batched ensemble shards naturally:
`shard_systems` assigns whole systems to ranks, largest first, each to the
rank with the fewest atoms so far, so every rank runs its own `Ensemble` and
nothing else is exchanged.

The reductions work with any initialised `torch.distributed` process group
(NCCL on GPUs, gloo on CPU) and are identities on a single process.
"""
from __future__ import annotations

import numpy as np

__all__ = ["world", "max_over_ranks", "sum_over_ranks", "shard_systems", "take_systems"]


def world():
    """(world_size, rank) of the initialised process group, else (1, 0)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist.get_world_size(), dist.get_rank()
    return 1, 0


def _reduce(value: float, op, device=None) -> float:
    import torch
    import torch.distributed as dist
    ws, _ = world()
    if ws == 1:
        return float(value)
    if device is None:
        device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value: float, device=None) -> float:
    """The largest value over all ranks (the job's time is its slowest rank's)."""
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.MAX, device)


def sum_over_ranks(value: float, device=None) -> float:
    """The sum over all ranks (work done by the whole job)."""
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.SUM, device)


def shard_systems(n_atoms, world_size: int) -> list[np.ndarray]:
    """Indices of the systems each rank runs: longest-processing-time-first
    greedy balance of the atom counts (ties to the lower rank; within a rank
    the systems keep their original order).  Every system goes to exactly one
    rank."""
    n_atoms = np.asarray(n_atoms, dtype=np.int64)
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    load = np.zeros(world_size, dtype=np.int64)
    owner = np.empty(len(n_atoms), dtype=np.int64)
    for k in np.argsort(-n_atoms, kind="stable"):
        r = int(np.argmin(load))
        owner[k] = r
        load[r] += n_atoms[k]
    return [np.flatnonzero(owner == r) for r in range(world_size)]


def take_systems(ens: dict, idx) -> dict:
    """The systems `idx` of an ensemble dict (per-system arrays indexed, the
    concatenated x and v cut to those systems' atoms, in `idx` order)."""
    idx = np.asarray(idx, dtype=np.int64)
    n = np.asarray(ens["n_atoms"], dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(n)])
    atoms = (np.concatenate([np.arange(off[k], off[k + 1]) for k in idx])
             if len(idx) else np.zeros(0, dtype=np.int64))
    out = {}
    for key, val in ens.items():
        if key in ("x", "v"):
            out[key] = np.asarray(val)[atoms]
        else:
            arr = np.asarray(val)
            out[key] = arr[idx] if arr.ndim >= 1 and len(arr) == len(n) else val
    return out
