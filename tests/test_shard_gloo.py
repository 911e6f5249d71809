"""Sharding the forward by pixel range across ranks (world size 2, gloo on
CPU): each rank traces its share with the oracle, the shards are all-gathered
and must equal the single-process full-sky maps bit for bit."""
import os
import socket

import numpy as np
import pytest

import srt_shard

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_ranges_cover_exactly():
    for count in (0, 1, 7, 48, 1000):
        for world in (1, 2, 3, 8):
            spans = [srt_shard.shard_range(5, count, r, world) for r in range(world)]
            pos = 5
            for b, c in spans:
                assert b == pos and c >= 0
                pos += c
            assert pos == 5 + count
            assert max(c for _, c in spans) - min(c for _, c in spans) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    import sys

    for p in (ROOT, os.path.join(ROOT, "snapshot-raytracer_gb300")):
        sys.path.insert(0, p)
    import torch.distributed as dist

    import srt_fields
    import srt_shard as sh
    from oracle import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    phi, b = srt_fields.int_noise_fields(16, seed=5)
    nside, steps, begin, count = 3, 9, 10, 83  # an odd range, uneven shards
    sb, sc = sh.shard_range(begin, count, rank, world)
    part = oracle.trace(phi, b, nside, steps, sb, sc, mode="fp64", threads=1)
    full = sh.gather_maps(part, begin, count)
    # timing reduction as bench.py does it: max over ranks
    import torch

    t = torch.tensor([float(rank + 1)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        np.save(out_path, full)
        assert t.item() == float(world)
    dist.destroy_process_group()


def test_two_rank_gloo_shards_match_single_process(tmp_path, orc):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import srt_fields

    out = str(tmp_path / "full.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    phi, b = srt_fields.int_noise_fields(16, seed=5)
    want = orc.trace(phi, b, 3, 9, 10, 83, mode="fp64")
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
