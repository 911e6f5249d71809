"""Sharding by pixel range across ranks (world size 2, gloo on CPU).
Forward: each rank traces its share with the oracle, the shards are
all-gathered and must equal the single-process full-sky maps bit for bit.
Adjoint: each rank takes its slice of the map weights; the sum all-reduce of
the ranks' derivatives (here the oracle's exact directional derivatives, the
gradient contracted with fixed directions) equals the single-process one."""
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


def _adj_worker(rank, world, port, out_path):
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
    phi, b = srt_fields.int_noise_fields(16, seed=6)
    nside, steps, begin, count = 2, 8, 3, 41
    w = np.random.default_rng(1).standard_normal((6, count)).astype(np.float32)
    rng = np.random.default_rng(2)
    dphi = [rng.standard_normal(phi.shape).astype(np.float32) for _ in range(2)]
    db = [rng.standard_normal(b.shape).astype(np.float32) for _ in range(2)]
    wr, br, cr = sh.shard_weights(w, begin, count, rank, world)
    L, dL = oracle.tangent(phi, b, nside, steps, np.arange(br, br + cr), wr, dphi, db, threads=1)
    red = sh.allreduce_gradients([np.array([L] + list(dL), np.float64)])[0]
    if rank == 0:
        np.save(out_path, red)
    dist.destroy_process_group()


def test_two_rank_gloo_adjoint_shards_sum_to_full(tmp_path, orc):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import srt_fields

    out = str(tmp_path / "adj.npy")
    mp.start_processes(_adj_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    phi, b = srt_fields.int_noise_fields(16, seed=6)
    w = np.random.default_rng(1).standard_normal((6, 41)).astype(np.float32)
    rng = np.random.default_rng(2)
    dphi = [rng.standard_normal(phi.shape).astype(np.float32) for _ in range(2)]
    db = [rng.standard_normal(b.shape).astype(np.float32) for _ in range(2)]
    L, dL = orc.tangent(phi, b, 2, 8, np.arange(3, 44), w, dphi, db)
    want = np.array([L] + list(dL))
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
