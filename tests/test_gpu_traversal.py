"""BVH traversal on the GPU against the oracle's independent BVH: closest
hits (t, instance, primitive, barycentrics) bit for bit, occlusion queries,
watertightness on shared edges and vertices, and the tmin/tmax contract."""
import numpy as np
import pytest

import asuna_gb300 as ag
from asuna_gb300 import scenes
from oracle import oracle_py

pytestmark = pytest.mark.gpu


def _random_rays(rng, n, center, radius):
    o = center + rng.normal(size=(n, 3)) * radius * 1.5
    tgt = center + rng.normal(size=(n, 3)) * radius * 0.5
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def test_closest_hit_matches_oracle(ctx):
    b, _ = scenes.mixed_scene(8, 8, frames=1, n_spheres=16, level=4, seed=5, env_size=(32, 16))
    d = b.desc()
    scene = ctx.create_scene(d)
    o_sc = oracle_py.OracleScene(d)
    rng = np.random.default_rng(0)
    o, dirs = _random_rays(rng, 4000, np.zeros(3), 10.0)
    hits, inst = scene.trace(o, dirs)
    mism = 0
    for k in range(len(o)):
        r = o_sc.trace(o[k], dirs[k])
        if r is None:
            mism += inst[k] != 0xFFFFFFFF
            continue
        t, ii, prim, u, v = r
        got = (hits[k, 0], inst[k], hits[k, 3].view(np.uint32), hits[k, 1], hits[k, 2])
        if not (got[0] == np.float32(t) and got[1] == ii and got[2] == prim and got[3] == np.float32(u)
                and got[4] == np.float32(v)):
            mism += 1
    # (closest hits resolve exact ties to the lowest instance and primitive
    # and both box tests are conservative, so none is expected; two of the
    # 4,000 are allowed)
    assert mism <= 2, mism


def test_occlusion_matches_oracle(ctx):
    b, _ = scenes.mixed_scene(8, 8, frames=1, n_spheres=16, level=3, seed=6, env_size=(32, 16))
    d = b.desc()
    scene = ctx.create_scene(d)
    o_sc = oracle_py.OracleScene(d)
    rng = np.random.default_rng(1)
    o, dirs = _random_rays(rng, 3000, np.zeros(3), 10.0)
    tmax = rng.uniform(0.5, 30.0, len(o)).astype(np.float32)
    hits, inst = scene.trace(o, dirs, tmin=0.0, tmax=tmax, any_hit=True)
    got = hits[:, 0] > 0
    want = np.array([o_sc.occluded(o[k], dirs[k], 0.0, float(tmax[k])) for k in range(len(o))])
    assert np.mean(got == want) >= 0.999


def test_watertight_shared_edges_and_vertices(ctx):
    # rays aimed exactly at vertices and edge midpoints of a closed icosphere never miss it
    v, f = scenes.icosphere(3)
    b = ag.SceneBuilder()
    m = b.add_lambertian("m", (0.5, 0.5, 0.5))
    verts = np.zeros(len(v), ag._abi.VERTEX_DTYPE)
    verts["pos"] = v.astype(np.float32)
    b.add_mesh("ico", verts, f.astype(np.uint32))
    b.add_instance("ico", m)
    scene = ctx.create_scene(b.desc())
    p = verts["pos"].astype(np.float64)
    targets = np.concatenate([p, 0.5 * (p[f[:, 0]] + p[f[:, 1]]), (p[f[:, 0]] + p[f[:, 1]] + p[f[:, 2]]) / 3])
    rng = np.random.default_rng(2)
    origins = rng.normal(size=targets.shape) * 0.05  # from inside the sphere
    dirs = targets - origins
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    hits, inst = scene.trace(origins.astype(np.float32), dirs.astype(np.float32), tmin=0.0)
    assert np.all(inst != 0xFFFFFFFF), int(np.sum(inst == 0xFFFFFFFF))


def test_watertight_tiled_plane_matches_oracle(ctx):
    # an irregular tiled plane (random diagonals, jittered interior vertices):
    # rays at random slants aimed at every vertex and edge midpoint all hit,
    # and hit what the oracle hits, bit for bit.  Each ray meets two or more
    # triangles at one point on the corner of their leaf boxes: both
    # traversals' box tests must keep every such box (both widen the far
    # distance by 2^-20) for the closest-hit choice to agree
    n = 12
    rng = np.random.default_rng(4)
    xs, ys = np.meshgrid(np.linspace(-1.0, 1.0, n + 1), np.linspace(-1.0, 1.0, n + 1), indexing="ij")
    pos = np.stack([xs, ys, np.zeros_like(xs)], axis=-1).reshape(-1, 3)
    inner = (np.abs(pos[:, 0]) < 0.999) & (np.abs(pos[:, 1]) < 0.999)
    pos[inner, :2] += rng.uniform(-0.3, 0.3, size=(int(inner.sum()), 2)) / n
    faces = []
    for i in range(n):
        for j in range(n):
            a, b_, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, (i + 1) * (n + 1) + j + 1, i * (n + 1) + j + 1
            faces += [(a, b_, c), (a, c, d)] if rng.random() < 0.5 else [(a, b_, d), (b_, c, d)]
    faces = np.array(faces)
    b = ag.SceneBuilder()
    m = b.add_lambertian("m", (0.5, 0.5, 0.5))
    verts = np.zeros(len(pos), ag._abi.VERTEX_DTYPE)
    verts["pos"] = pos.astype(np.float32)
    b.add_mesh("plane", verts, faces.astype(np.uint32))
    b.add_instance("plane", m)
    d = b.desc()
    scene = ctx.create_scene(d)
    o_sc = oracle_py.OracleScene(d)
    p = verts["pos"].astype(np.float64)
    edges = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    targets = np.concatenate([p[inner], 0.5 * (p[edges[:, 0]] + p[edges[:, 1]])])
    targets = targets[(np.abs(targets[:, 0]) < 0.99) & (np.abs(targets[:, 1]) < 0.99)]
    slant = rng.uniform(-0.6, 0.6, size=(len(targets), 2))
    origins = (targets + np.column_stack([slant, np.ones(len(targets))])).astype(np.float32)
    dirs = (targets - origins)
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    hits, inst = scene.trace(origins, dirs, tmin=0.0)
    assert np.all(inst != 0xFFFFFFFF), int(np.sum(inst == 0xFFFFFFFF))
    same = 0
    for k in range(len(origins)):
        t, ii, prim, u, v = o_sc.trace(origins[k], dirs[k], 0.0, 1e10)
        same += (hits[k, 0] == np.float32(t) and hits[k, 3].view(np.uint32) == prim and
                 hits[k, 1] == np.float32(u) and hits[k, 2] == np.float32(v))
    assert same == len(origins), (same, len(origins))


def test_tmin_tmax_contract(ctx):
    b, _ = scenes.box_scene(8, 8, frames=1)
    scene = ctx.create_scene(b.desc())
    o = np.array([[0.5, 0.5, 0.0]] * 3, np.float32)
    dirs = np.array([[0.0, 0.0, -1.0]] * 3, np.float32)  # back wall at z = -1 (t = 1), above both cuboids
    hits, inst = scene.trace(o, dirs, tmin=0.0, tmax=np.float32(1e10))
    assert np.allclose(hits[:, 0], 1.0)
    occ, _ = scene.trace(o, dirs, tmin=0.0, tmax=np.float32(0.999), any_hit=True)
    assert np.all(occ[:, 0] < 0)
    occ, _ = scene.trace(o, dirs, tmin=0.0, tmax=np.float32(1.001), any_hit=True)
    assert np.all(occ[:, 0] > 0)
    hits, inst = scene.trace(o, dirs, tmin=1.5, tmax=np.float32(1e10))
    assert np.all(inst == 0xFFFFFFFF)


def test_truncated_traversal_is_reported(ctx):
    """A traversal cut short by a full stack makes every render entry point
    fail with ERR_TRAVERSAL: the call itself when it waits (stats, records),
    else the next call that waits (film read, sync).  Each cut is reported
    once, and the context renders normally afterwards."""
    from asuna_gb300 import _abi as A

    b, shot = scenes.box_scene(32, 32, frames=1, max_depth=3)
    scene = ctx.create_scene(b.desc())
    film = ctx.create_film(32, 32)
    try:
        ctx.set_traversal_stack(1)  # entering any instance needs a second entry
        ctx.render(scene, shot, film)  # asynchronous: queued without error
        with pytest.raises(A.AsunaError) as e:
            film.read(0)
        assert e.value.code == A.ERR_TRAVERSAL
        with pytest.raises(A.AsunaError) as e:
            ctx.render(scene, shot, film, stats=True)
        assert e.value.code == A.ERR_TRAVERSAL
        with pytest.raises(A.AsunaError) as e:
            ctx.render_paths(scene, shot, film)
        assert e.value.code == A.ERR_TRAVERSAL
        ctx.render(scene, shot, film)
        with pytest.raises(A.AsunaError) as e:
            ctx.sync()
        assert e.value.code == A.ERR_TRAVERSAL
    finally:
        ctx.set_traversal_stack(0)
    ctx.render(scene, shot, film, stats=True)
    film.read(0)
    ctx.sync()


def test_runaway_traversal_is_reported(ctx):
    """A ray that would walk past the traversal's loop bound (70,000
    coincident instances) is stopped and reported, not left running."""
    from asuna_gb300 import _abi as A

    b, shot = scenes.stacked_instances_scene(70000)
    scene = ctx.create_scene(b.desc())
    film = ctx.create_film(shot.width, shot.height)
    with pytest.raises(A.AsunaError) as e:
        ctx.render(scene, shot, film, stats=True)
    assert e.value.code == A.ERR_TRAVERSAL
    # a few hundred copies stay far inside the bound
    b2, shot2 = scenes.stacked_instances_scene(300)
    scene2 = ctx.create_scene(b2.desc())
    ctx.render(scene2, shot2, film, stats=True)
    assert float(film.read(0)[..., :3].max()) > 0.0


def test_device_bvh_build_matches_host_build(ctx):
    """The bottom-level BVHs built on the device (the default) and on host
    threads run the same binned-SAH algorithm: every closest hit and every
    occlusion answer of 20,000 random rays is identical, and the trees are
    of the same size and depth class."""
    b, _ = scenes.mixed_scene(8, 8, frames=1, n_spheres=24, level=5, seed=9, env_size=(32, 16))
    d = b.desc()
    dev = ctx.create_scene(d)
    ctx.set_bvh_build(on_device=False)
    try:
        host = ctx.create_scene(d)
    finally:
        ctx.set_bvh_build(on_device=True)
    rng = np.random.default_rng(3)
    o, dirs = _random_rays(rng, 20000, np.zeros(3), 10.0)
    for any_hit in (False, True):
        h1, i1 = dev.trace(o, dirs, any_hit=any_hit)
        h2, i2 = host.trace(o, dirs, any_hit=any_hit)
        assert np.array_equal(i1, i2)
        assert np.array_equal(h1.view(np.uint32), h2.view(np.uint32))
    s1, s2 = dev.stats(), host.stats()
    assert s1["triangles"] == s2["triangles"]
    # the same algorithm: node counts within a few percent (chunked allocation aside)
    assert abs(s1["blas_nodes"] - s2["blas_nodes"]) <= 0.05 * s2["blas_nodes"] + 64 * 256


@pytest.mark.parametrize("n_tris", [1, 3, 4, 5, 2049, 70000])
def test_device_bvh_build_edge_sizes(ctx, n_tris):
    """Single meshes around the builder's thresholds (one triangle, a leaf,
    one above a leaf, one above a warp's subtree, many) plus coincident
    triangles: device and host builds give identical hits."""
    from asuna_gb300 import _abi as A

    rng = np.random.default_rng(n_tris)
    b = ag.SceneBuilder()
    m = b.add_lambertian("m", (0.5, 0.5, 0.5))
    p = rng.uniform(-1, 1, (n_tris, 3)).astype(np.float32)
    p[: n_tris // 4] = 0.25  # a quarter of the triangles share one place
    v = np.zeros(3 * n_tris, A.VERTEX_DTYPE)
    v["pos"] = (p[:, None, :] + rng.uniform(-0.05, 0.05, (n_tris, 3, 3)).astype(np.float32)).reshape(-1, 3)
    v["pos"][: 3 * (n_tris // 4)] = np.tile(np.array([[0.2, 0.2, 0.2], [0.3, 0.2, 0.2], [0.2, 0.3, 0.2]],
                                                     np.float32), (n_tris // 4, 1))
    v["normal"] = (0, 0, 1)
    b.add_mesh("t", v, np.arange(3 * n_tris, dtype=np.uint32))
    b.add_instance("t", m)
    b.add_instance("t", m, np.array([[1, 0, 0, 3], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32))
    d = b.desc()
    dev = ctx.create_scene(d)
    ctx.set_bvh_build(on_device=False)
    try:
        host = ctx.create_scene(d)
    finally:
        ctx.set_bvh_build(on_device=True)
    o, dirs = _random_rays(rng, 4000, np.array([1.5, 0.0, 0.0]), 2.0)
    # half of the rays aim at triangle centres (of either instance)
    tc = v["pos"].reshape(-1, 3, 3).mean(1)[rng.integers(0, n_tris, 2000)] + \
        np.array([3.0, 0.0, 0.0], np.float32) * rng.integers(0, 2, (2000, 1))
    dd = tc - o[:2000]
    dirs[:2000] = (dd / np.linalg.norm(dd, axis=1, keepdims=True)).astype(np.float32)
    h1, i1 = dev.trace(o, dirs)
    h2, i2 = host.trace(o, dirs)
    assert np.array_equal(i1, i2)
    assert np.array_equal(h1.view(np.uint32), h2.view(np.uint32))
    assert (i1 != 0xFFFFFFFF).sum() > 0
