"""Autotuner coordinate search on a fake context (host logic only, no GPU).

The fake context times a render from a synthetic throughput surface over the
launch settings; the tuner must land on its optimum, leave the context set to
it, and give the shot back its own frame range."""
import types

from asuna_gb300 import autotune


class FakeCtx:
    def __init__(self, score):
        self.score = score
        self.trav = None
        self.launch = None
        self.sort = None
        self.budget = None
        self.shape = (0, 0)
        self.renders = []

    def set_traversal(self, *t):
        self.trav = tuple(t)
        self.shadow_occ = t[4] if len(t) > 4 else 0

    def set_traversal_occupancy(self, extend, shadow):
        self.trav = self.trav[:4] + (extend,)
        self.shadow_occ = shadow

    def set_launch(self, t, s):
        self.launch = (t, s)

    def set_ray_sort(self, m):
        self.sort = m

    def set_traversal_shape(self, threads=0, shared=0):
        self.shape = (threads, shared)

    def set_path_budget(self, b):
        self.budget = b

    def render(self, scene, shot, film, stats=False):
        self.renders.append((shot.frame0, shot.frames))
        mrays = self.score(shot.frames, self.launch, self.trav, self.sort) + \
            {(0, 0): 0, (128, 32): 4, (64, 24): -2, (256, 24): 1, (128, 16): -1}[self.shape] + \
            {8: 0, 10: 1, 12: 2}[self.shadow_occ] - {8: 0, 10: 1, 12: 2}[self.trav[4]]
        rays = 1e6
        return {"extend_rays": rays, "shadow_rays": 0, "ms_total": rays / (mrays * 1e3)}


class FakeFilm:
    def __init__(self):
        self.cleared = 0

    def clear(self):
        self.cleared += 1


def _score(frames, launch, trav, sort):
    # best: 16 frames, default grids, occupancy 10, extend refill 24 only
    # when sorted (8 unsorted), shadow refill 4, speculation on, sort mode 3
    v = 1000.0 - abs(frames - 16) - 5 * (launch != (0, 0))
    v -= 3 * abs(trav[4] - 10)
    want_ext = 24 if sort else 8
    v -= 0.5 * abs(trav[0] - want_ext)
    v -= 0.5 * abs(trav[1] - 4)
    v += 2 * trav[2] + trav[3]
    v += {0: 0, 1: 10, 2: 15, 3: 20}[sort]
    return v


def test_tune_finds_the_optimum_and_restores_the_shot():
    ctx = FakeCtx(_score)
    shot = types.SimpleNamespace(width=64, height=32, frame0=5, frames=3)
    film = FakeFilm()
    best = autotune.tune(ctx, object(), shot, film, memory_bytes=1 << 40)
    assert best["frames"] == 16
    assert (best["trace_blocks_per_sm"], best["shade_blocks_per_sm"]) == (0, 0)
    assert best["ray_sort"] == 3
    # the extend refill is tuned again once the sort is on
    assert best["traversal"] == (24, 4, 1, 1, 10)
    assert ctx.trav == best["traversal"] and ctx.sort == 3 and ctx.launch == (0, 0)
    # block shape and shared stack depth: 128 threads, 32 entries
    assert best["shape"] == (128, 32) and ctx.shape == (128, 32)
    # the occlusion pass's own kernel variant
    assert best["shadow_occupancy"] == 12 and ctx.shadow_occ == 12 and ctx.trav[4] == 10
    assert ctx.budget == 16 * 64 * 32 * autotune.BYTES_PER_PATH
    assert (shot.frame0, shot.frames) == (5, 3) and film.cleared == 1
    # tuning frames never overlap the caller's sample streams
    assert all(f0 >= 1 << 20 for f0, _ in ctx.renders)
    assert len(best["trials"]) > 10


def test_tune_respects_the_memory_bound():
    ctx = FakeCtx(_score)
    shot = types.SimpleNamespace(width=64, height=32, frame0=0, frames=1)
    best = autotune.tune(ctx, object(), shot, FakeFilm(), memory_bytes=4 * 64 * 32 * autotune.BYTES_PER_PATH)
    assert best["frames"] == 4


def test_tune_skips_wavefronts_that_do_not_fit():
    """A frame count whose wavefront does not fit in the device memory left
    (ERR_OOM from the render) ends the frame sweep; the tuner keeps the best
    count that rendered."""
    from asuna_gb300._abi import ERR_OOM, AsunaError

    class OomCtx(FakeCtx):
        def render(self, scene, shot, film, stats=False):
            if shot.frames > 8:
                raise AsunaError(ERR_OOM, "wavefront buffers do not fit")
            return super().render(scene, shot, film, stats)

    ctx = OomCtx(_score)
    shot = types.SimpleNamespace(width=64, height=32, frame0=5, frames=3)
    best = autotune.tune(ctx, object(), shot, FakeFilm(), memory_bytes=1 << 40)
    assert best["frames"] == 8
    assert any(t.get("error") == "out of memory" and t["frames"] == 16 for t in best["trials"])
    assert not any(t.get("frames") == 32 for t in best["trials"] if "trace" in t)
    assert (shot.frame0, shot.frames) == (5, 3)
