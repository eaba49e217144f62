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


def _shard_case():
    """A ragged table with a heightmap, upstream gradients over its output
    vertices, and the texels (all seeded, identical in every process)."""
    import types
    from oracle import oracle as O
    from wave_tool_gb300 import workloads
    w = workloads.small_random(31, n_patches=9, side_range=(2, 60), n_waves_range=(1, 12))
    tex = O.noise_f64(w.heightmap.terms, w.heightmap.width, w.heightmap.height).astype(np.float32)
    hmp = types.SimpleNamespace(sample_scale=w.heightmap.sample_scale, disp_scale=w.heightmap.disp_scale,
                                wrap=w.heightmap.wrap)
    rng = np.random.default_rng(5)
    gpos = rng.standard_normal((w.n_vertices, 4)).astype(np.float32)
    gnrm = rng.standard_normal((w.n_vertices, 4)).astype(np.float32)
    return w, tex, hmp, gpos, gnrm


def _rows_of(patches):
    """Output index ranges of each patch, in table order."""
    return [np.arange(int(p["out_offset"]), int(p["out_offset"]) + int(p["cols"]) * int(p["rows"]))
            for p in patches]


def _shard_worker(rank, world, port, q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "tests"))
    import __graft_entry__
    __graft_entry__.load_package()
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    from wave_tool_gb300 import fit, sharding
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, tex, hmp, gpos, gnrm = _shard_case()
    mine, idx = sharding.shard_patches(w.patches, world, rank)
    # this rank's outputs with the CPU restatement of the shader
    _, pos4, nrm4 = O.cpu_baseline(mine, w.waves, tex, hmp, threads=1)
    # this rank's slice of the upstream gradients, in its dense output order
    src = np.concatenate(_rows_of(w.patches[idx])) if len(idx) else np.zeros(0, np.int64)
    g64 = O.adjoint_f64(mine, w.waves, gpos[src], gnrm[src], tex, hmp) if len(idx) else np.zeros((len(w.waves), 8))
    g = fit.rank_sum(torch.from_numpy(g64.astype(np.float32)), dist.group.WORLD)
    parts = [None] * world
    dist.all_gather_object(parts, (idx.tolist(), pos4, nrm4))
    if rank == 0:
        q.put((g.numpy(), g64, parts))
    else:
        q.put((g.numpy(), g64, None))
    dist.destroy_process_group()


def test_two_rank_shards_recombine_to_the_one_rank_outputs_and_gradients():
    """The split of one table over two ranks (LPT shards of its patches):
    each rank's CPU-restatement outputs, put back at their patches' output
    offsets, equal the one-rank outputs bit for bit; the rank-ordered sum of
    the ranks' FP32 wave gradients (FP64 closed forms on each shard) equals
    the one-rank gradient to FP32 rounding, and is the same on both ranks."""
    import torch.multiprocessing as mp
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    from oracle import build, oracle as O
    build.build_oracle()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    w, tex, hmp, gpos, gnrm = _shard_case()
    _, pos_full, nrm_full = O.cpu_baseline(w.patches, w.waves, tex, hmp, threads=1)
    g_full = O.adjoint_f64(w.patches, w.waves, gpos, gnrm, tex, hmp)
    parts = next(r[2] for r in res if r[2] is not None)
    pos = np.full_like(pos_full, np.nan)
    nrm = np.full_like(nrm_full, np.nan)
    seen = []
    for idx, p4, n4 in parts:
        seen += idx
        o = 0
        for i in idx:   # the rank's patches in its dense order
            r = _rows_of(w.patches[i:i + 1])[0]
            pos[r] = p4[o:o + len(r)]
            nrm[r] = n4[o:o + len(r)]
            o += len(r)
    assert sorted(seen) == list(range(len(w.patches)))
    assert np.array_equal(pos, pos_full) and np.array_equal(nrm, nrm_full)
    g0, g1 = res[0][0], res[1][0]
    assert np.array_equal(g0, g1)  # every rank holds the same bits
    # rank-ordered FP32 sum vs the one-rank FP64 gradient rounded to FP32
    mag = np.abs(res[0][1]) + np.abs(res[1][1])
    assert np.all(np.abs(g0.astype(np.float64) - g_full) <= 4 * np.finfo(np.float32).eps * mag + 1e-30)
