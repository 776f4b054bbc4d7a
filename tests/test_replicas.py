"""Replica sharding (no GPU): frame and shot shards cover the work exactly
once, and two gloo ranks agree on the combined result."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from asuna_gb300 import replicas


@pytest.mark.parametrize("world,frames", [(1, 7), (2, 7), (3, 64), (8, 5)])
def test_frame_shards_partition(world, frames):
    seen = []
    for r in range(world):
        b, n = replicas.frame_shard(r, world, 10, frames)
        seen += list(range(b, b + n))
    assert seen == list(range(10, 10 + frames))


def test_shot_shards_partition():
    got = sorted(i for r in range(3) for i in replicas.shot_shard(r, 3, 10))
    assert got == list(range(10))


def test_merge_equals_running_mean():
    rng = np.random.default_rng(0)
    samples = rng.uniform(0, 5, size=(6, 4, 4, 3)).astype(np.float32)
    w = rng.uniform(0.5, 1.0, size=(6, 4, 4, 1)).astype(np.float32)
    full = (samples * w).sum(0) / w.sum(0)
    parts = []
    for a, b in ((0, 2), (2, 6)):
        r = (samples[a:b] * w[a:b]).sum(0) / w[a:b].sum(0)
        parts.append((np.concatenate([r, np.ones_like(r[..., :1])], -1), np.repeat(w[a:b].sum(0), 4, -1)))
    out, ws = replicas.merge_films(parts)
    assert np.allclose(out[..., :3], full, rtol=1e-5)
    assert np.allclose(ws, w.sum(0)[..., 0], rtol=1e-6)


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch

    b, n = replicas.frame_shard(rank, world, 0, 9)
    local = torch.tensor([float(n), float(b)], dtype=torch.float64)
    total = local.clone()
    dist.all_reduce(total, op=dist.ReduceOp.SUM)
    mx = torch.tensor([float(rank + 1)], dtype=torch.float64)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    q.put((rank, int(total[0]), float(mx[0])))
    dist.destroy_process_group()


def test_two_gloo_ranks_cover_all_frames():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [o[1] for o in out] == [9, 9] and [o[2] for o in out] == [2.0, 2.0]


def _render_worker(rank, world, port, q):
    """Renders this rank's frames of the small box scene with the CPU oracle
    and sends (radiance, weight sum) to rank 0, which merges them."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from asuna_gb300 import scenes
    from oracle import oracle_py

    b, shot = scenes.box_scene(24, 20, frames=10, max_depth=5)
    first, count = replicas.frame_shard(rank, world, 0, shot.frames)
    shot.frame0, shot.frames = first, count
    film, _, _ = oracle_py.OracleScene(b.desc()).render(shot, records=False)
    parts = [None] * world
    dist.all_gather_object(parts, (film[0], film[8]))
    if rank == 0:
        merged, wsum = replicas.merge_films(parts)
        q.put((merged, wsum))
    dist.destroy_process_group()


def test_two_gloo_ranks_render_and_merge_like_one_process():
    """Two ranks render disjoint frame shards (the CPU oracle stands in for
    each rank's GPU); the merged film equals a single-process render of all
    frames.  The single process keeps the reference's float32 running mean
    frame by frame (rgen:171-178); the merge sums the two shards' weighted
    means in float64, so the two agree to float32 rounding (1e-5 relative),
    and the weight sums exactly up to float32 summation order."""
    from asuna_gb300 import scenes
    from oracle import oracle_py

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29700 + os.getpid() % 1000
    procs = [ctx.Process(target=_render_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged, wsum = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
    b, shot = scenes.box_scene(24, 20, frames=10, max_depth=5)
    film, _, _ = oracle_py.OracleScene(b.desc()).render(shot, records=False)
    assert np.allclose(merged[..., :3], film[0][..., :3], rtol=1e-5, atol=1e-7)
    assert np.allclose(wsum, film[8][..., 0], rtol=1e-6)
    assert float(film[0][..., :3].mean()) > 0.0
