"""Multi-process host logic of the N > 1 paths, on CPU with gloo (world size 2)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from tensorfox_gb300.distributed import cpd_batch_distributed, max_over_ranks, shard_bounds


def test_shard_bounds_cover_in_order():
    for n in (0, 1, 5, 7, 4096):
        for world in (1, 2, 3, 8):
            got = [shard_bounds(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _fake_solve(tensors, ranks, options):
    # stands in for the GPU batch solver: one record per problem
    return [(float(np.sum(t)), int(r), dist.get_rank()) for t, r in zip(tensors, ranks)]


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(0)   # same problems on every rank
        Ts = [rng.standard_normal((3, 4, 5)) for _ in range(7)]
        Rs = [int(r) for r in rng.integers(2, 6, size=7)]
        res = cpd_batch_distributed(Ts, Rs, None, solve=_fake_solve)
        m = max_over_ranks([1.0 + rank, 10.0 - rank])
        torch.save({"res": res, "max": m}, os.path.join(out_dir, "r%d.pt" % rank))
    finally:
        dist.destroy_process_group()


def test_batch_sharding_and_timing_max_world2(tmp_path):
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    outs = [torch.load(os.path.join(str(tmp_path), "r%d.pt" % r), weights_only=False) for r in range(world)]
    rng = np.random.default_rng(0)
    Ts = [rng.standard_normal((3, 4, 5)) for _ in range(7)]
    Rs = [int(r) for r in rng.integers(2, 6, size=7)]
    for o in outs:
        res = o["res"]
        assert len(res) == 7
        # original order, each problem solved exactly once, by the rank owning its slice
        for i, (s, r, owner) in enumerate(res):
            assert s == pytest.approx(float(np.sum(Ts[i])))
            assert r == Rs[i]
            lo, hi = shard_bounds(7, owner, world)
            assert lo <= i < hi
        assert o["max"] == [2.0, 10.0]
    assert outs[0]["res"] == outs[1]["res"]
