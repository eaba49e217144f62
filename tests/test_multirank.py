"""Multi-rank logic on CPU: world_size-2 gloo process groups (no GPU)."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    import __graft_entry__
    __graft_entry__.load_package()
    import torch
    import torch.distributed as dist
    from wave_tool_gb300 import sharding, workloads
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = workloads.config3(n_patches=40, seed=3)
    mine, idx = sharding.shard_patches(w.patches, world, rank)
    terms = int(np.sum(mine["cols"].astype(np.int64) * mine["rows"] * mine["wave_count"]))
    t = torch.tensor([terms, len(idx)], dtype=torch.int64)
    dist.all_reduce(t)
    ids = [None] * world
    dist.all_gather_object(ids, idx.tolist())
    # per-rank "gradients": deterministic per rank, summed in rank order
    g = torch.arange(12, dtype=torch.float32).reshape(3, 4) * (rank + 1) + 0.1 * rank
    s1 = sharding.allreduce_grads_fixed_order(g)
    s2 = sharding.allreduce_grads_fixed_order(g)
    q.put((rank, int(t[0]), int(t[1]), ids, s1.numpy(), bool(torch.equal(s1, s2)), mine["out_offset"].tolist(),
           (mine["cols"].astype(np.int64) * mine["rows"]).tolist()))
    dist.destroy_process_group()


def test_two_rank_sharding_and_fixed_order_reduction():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted([q.get(timeout=120) for _ in procs])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    from wave_tool_gb300 import workloads
    w = workloads.config3(n_patches=40, seed=3)
    total = int(np.sum(w.patches["cols"].astype(np.int64) * w.patches["rows"] * w.patches["wave_count"]))
    r0, r1 = out
    assert r0[1] == r1[1] == total and r0[2] == 40
    assert sorted(r0[3][0] + r0[3][1]) == list(range(40))            # every patch on exactly one rank
    # LPT balance: the larger share is within the largest patch of the smaller
    exp = np.arange(12, dtype=np.float32).reshape(3, 4) * 3 + 0.1
    assert np.array_equal(r0[4], r1[4]) and np.allclose(r0[4], exp)
    assert r0[5] and r1[5]
    for r in out:  # dense per-rank output offsets
        offs, sizes = r[6], r[7]
        assert offs == list(np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(int))
