"""Replica sharding of render work across GPUs (one process per GPU).

The path shards with no data exchange: shots, frames and requests are
independent.  Every rank renders its own frames (or shots); results are only
combined on the host, and a film split by frames is recombined with the
reference's running weighted mean (src/shaders/raytrace.projective.rgen:171-178)
in frame order, which is what merge_films() does.
"""
import numpy as np


def frame_shard(rank, world, frame0, frames):
    """Contiguous frames [begin, begin + count) of rank `rank` out of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(frames, world)
    begin = frame0 + rank * base + min(rank, extra)
    return begin, base + (1 if rank < extra else 0)


def shot_shard(rank, world, nshots):
    """Shot indices of rank `rank` (round robin)."""
    return list(range(rank, nshots, world))


def merge_films(parts):
    """Combine (radiance, weight) images of consecutive frame shards, in order:
    sum of weighted radiance over sum of weights, per pixel."""
    rad = None
    wsum = None
    for r, w in parts:
        if rad is None:
            rad = r[..., :3].astype(np.float64) * w[..., :1]
            wsum = w[..., :1].astype(np.float64).copy()
        else:
            rad += r[..., :3] * w[..., :1]
            wsum += w[..., :1]
    out = np.ones(rad.shape[:-1] + (4,), np.float32)
    out[..., :3] = rad / np.maximum(wsum, 1e-30)
    return out, wsum[..., 0]
