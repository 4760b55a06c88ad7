"""Multi-process (N > 1) host logic on CPU: two gloo ranks on 127.0.0.1.

The hot path runs as independent replicas (one engine per GPU, no exchange
step); what crosses ranks is host-side: the max-over-ranks timing and the
summed work that bench.py reports, and the assignment of an ensemble's
systems to ranks.  These run here as world_size-2 gloo process groups.
"""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, sizes, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        from naivedynamics import replicas
        assert replicas.world() == (ws, rank)
        # each rank's "time" and "work": the job's time is the slowest rank's
        t = replicas.max_over_ranks(1.5 + rank)
        w = replicas.sum_over_ranks(100.0 * (rank + 1))
        shards = replicas.shard_systems(sizes, ws)
        mine = shards[rank]
        atoms = replicas.sum_over_ranks(float(np.asarray(sizes)[mine].sum()))
        q.put((rank, t, w, [list(map(int, s)) for s in shards], atoms))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ws = 2
    sizes = [16324, 256, 4096, 1024, 8192, 512, 300, 2048, 9000, 777]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, sizes, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    for rank, t, w, shards, atoms in out:
        assert t == 2.5                      # max of 1.5, 2.5
        assert w == 300.0                    # 100 + 200
        assert shards == out[0][3]           # every rank computes the same assignment
        assert atoms == float(sum(sizes))    # every system runs exactly once
    _ = torch


def test_shard_systems_balance():
    from naivedynamics import replicas
    rng = np.random.default_rng(5)
    sizes = 4 * np.round(np.exp(rng.uniform(np.log(256), np.log(16384), 512)) / 4).astype(int)
    for ws in (1, 2, 4, 8):
        shards = replicas.shard_systems(sizes, ws)
        owned = np.sort(np.concatenate(shards))
        assert np.array_equal(owned, np.arange(len(sizes)))
        loads = np.array([sizes[s].sum() for s in shards])
        # greedy LPT: no rank exceeds the mean by more than the largest system
        assert loads.max() - loads.mean() <= sizes.max()
        for s in shards:
            assert np.all(np.diff(s) > 0)
    with pytest.raises(ValueError):
        replicas.shard_systems(sizes, 0)


def test_take_systems():
    from naivedynamics import replicas, synth
    e = synth.ensemble(7, nsys=6, nmin=256, nmax=1024)
    shards = replicas.shard_systems(e["n_atoms"], 2)
    parts = [replicas.take_systems(e, s) for s in shards]
    assert sum(len(p["n_atoms"]) for p in parts) == 6
    off = np.concatenate([[0], np.cumsum(e["n_atoms"])])
    for s, p in zip(shards, parts):
        assert len(p["x"]) == int(e["n_atoms"][s].sum()) == len(p["v"])
        at = 0
        for k in s:  # each system's atoms, in shard order
            n = int(e["n_atoms"][k])
            assert np.array_equal(p["x"][at:at + n], e["x"][off[k]:off[k] + n])
            assert p["sigma"][list(s).index(k)] == e["sigma"][k]
            at += n


def test_single_process_is_identity():
    from naivedynamics import replicas
    assert replicas.world() == (1, 0)
    assert replicas.max_over_ranks(3.25) == 3.25
    assert replicas.sum_over_ranks(7.0) == 7.0
