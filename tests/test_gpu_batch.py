"""Batching invariance: a shot's film is the same rendered alone, inside a
multi-shot wavefront, split across calls (resume from frame0), or through a
small path budget that forces many wavefront batches.  Seeds derive from
(pixel, frame, shot seed), never from queue slot or batch order."""
import numpy as np
import pytest

from asuna_gb300 import scenes

pytestmark = pytest.mark.gpu


def _film(ctx, scene, shot):
    f = ctx.create_film(shot.width, shot.height)
    ctx.render(scene, shot, f)
    return np.stack([f.read(k) for k in range(9)])


def test_batch_equals_alone(ctx):
    b, s1 = scenes.plugin_scene(64, 48, frames=3, max_depth=6)
    _, s2 = scenes.plugin_scene(40, 40, frames=5, max_depth=4, opencv=True)
    s2.seed = 7
    scene = ctx.create_scene(b.desc())
    a1, a2 = _film(ctx, scene, s1), _film(ctx, scene, s2)
    f1, f2 = ctx.create_film(64, 48), ctx.create_film(40, 40)
    ctx.render_batch(scene, [s1, s2], [f1, f2])
    assert np.array_equal(np.stack([f1.read(k) for k in range(9)]), a1)
    assert np.array_equal(np.stack([f2.read(k) for k in range(9)]), a2)


def test_resume_equals_single_call(ctx):
    b, shot = scenes.box_scene(48, 48, frames=8, max_depth=6)
    scene = ctx.create_scene(b.desc())
    full = _film(ctx, scene, shot)
    f = ctx.create_film(48, 48)
    shot.frames = 3
    ctx.render(scene, shot, f)
    shot.frame0, shot.frames = 3, 5
    ctx.render(scene, shot, f)
    assert np.array_equal(np.stack([f.read(k) for k in range(9)]), full)


def test_small_budget_many_batches(ctx):
    b, shot = scenes.box_scene(64, 64, frames=6, max_depth=6)
    scene = ctx.create_scene(b.desc())
    full = _film(ctx, scene, shot)
    ctx.set_path_budget(64 * 64 * 200)  # about one frame per wavefront
    try:
        small = _film(ctx, scene, shot)
    finally:
        ctx.set_path_budget(0)
    assert np.array_equal(small, full)


def test_seed_changes_streams(ctx):
    b, shot = scenes.box_scene(32, 32, frames=2, max_depth=4)
    scene = ctx.create_scene(b.desc())
    a = _film(ctx, scene, shot)
    shot.seed = 99
    c = _film(ctx, scene, shot)
    assert not np.array_equal(a[0], c[0])
    assert abs(float(a[0, ..., :3].mean()) - float(c[0, ..., :3].mean())) < 0.1


def test_graph_replay_equals_direct_launches(ctx):
    b, shot = scenes.plugin_scene(64, 48, frames=2, max_depth=6)
    scene = ctx.create_scene(b.desc())
    films = []
    for graphs in (False, True):
        ctx.set_graphs(graphs)
        f = ctx.create_film(64, 48)
        for k in range(3):  # the second and third calls replay the captured graph
            shot.frame0 = 2 * k
            ctx.render(scene, shot, f, stats=(k == 2))
        films.append(np.stack([f.read(i) for i in range(9)]))
    ctx.set_graphs(True)
    assert np.array_equal(films[0], films[1])


def test_traversal_settings_do_not_change_results(ctx):
    """Refill thresholds, speculative walking and the kernel variant
    (occupancy, block size, shared-memory stack entries) change the visiting
    order only: closest hits (ties to the lowest instance /
    primitive) and occlusion answers are the same, so films are
    bit-identical."""
    b, shot = scenes.plugin_scene(64, 48, frames=2, max_depth=6)
    scene = ctx.create_scene(b.desc())
    films = []
    for trav, shape in (((8, 8, 1, 1, 8), (0, 0)), ((1, 32, 0, 0, 10), (64, 16)), ((32, 1, 1, 0, 12), (256, 32)),
                        ((4, 16, 0, 1, 10), (128, 32)), ((24, 8, 1, 1, 10), (64, 32)), ((24, 8, 1, 1, 12), (256, 16))):
        ctx.set_traversal(*trav)
        ctx.set_traversal_shape(*shape)
        f = ctx.create_film(64, 48)
        ctx.render(scene, shot, f)
        films.append(np.stack([f.read(i) for i in range(9)]))
    ctx.set_traversal()
    ctx.set_traversal_shape()
    for f in films[1:]:
        assert np.array_equal(films[0], f)
    # the two passes on different kernel variants
    for ext, sh in ((8, 12), (12, 8), (10, 10)):
        ctx.set_traversal_occupancy(ext, sh)
        f = ctx.create_film(64, 48)
        ctx.render(scene, shot, f)
        assert np.array_equal(films[0], np.stack([f.read(i) for i in range(9)]))
    ctx.set_traversal()


def test_film_image_tensor_is_the_film(ctx):
    """asuna_film_image: a zero-copy device view equal to what film_read copies out."""
    b, shot = scenes.box_scene(40, 24, frames=2, max_depth=4, channels=("albedo", "normal"))
    scene = ctx.create_scene(b.desc())
    f = ctx.create_film(40, 24)
    ctx.render(scene, shot, f)
    ctx.sync()
    for k in (0, 1, 2, 8):
        t = f.tensor(k)
        assert t.shape == (24, 40, 4) and t.is_cuda
        assert np.array_equal(t.cpu().numpy(), f.read(k))


def test_ray_sort_does_not_change_results(ctx):
    """Sorting the extend queue reorders rays only: films (and per-path
    records) are bit-identical with and without it, including opacity
    pass-through and textured materials."""
    b, shot = scenes.plugin_scene(64, 48, frames=3, max_depth=8, textured=True, opacity=True)
    scene = ctx.create_scene(b.desc())
    out = []
    for mode in (0, 1, 2, 3):
        ctx.set_ray_sort(mode)
        f = ctx.create_film(64, 48)
        rec = ctx.render_paths(scene, shot, f)
        f2 = ctx.create_film(64, 48)
        ctx.render(scene, shot, f2)
        out.append((np.stack([f.read(i) for i in range(9)]), rec, np.stack([f2.read(i) for i in range(9)])))
    ctx.set_ray_sort(0)
    for imgs, rec, imgs2 in out[1:]:
        assert np.array_equal(out[0][0], imgs) and np.array_equal(out[0][1], rec)
        assert np.array_equal(out[0][2], imgs2)
