"""The oracle's ray/triangle test is watertight (host only, no GPU): rays
aimed exactly at the shared vertices and edges of closed or tiled meshes
never slip between triangles.  The GPU's traversal runs the same test with
the same rounding (tests/test_gpu_traversal.py compares the two bit for bit
and repeats the icosphere case on the device)."""
import numpy as np

import asuna_gb300 as ag
from asuna_gb300 import scenes
from oracle import oracle_py


def _scene(verts_pos, faces):
    b = ag.SceneBuilder()
    m = b.add_lambertian("m", (0.5, 0.5, 0.5))
    verts = np.zeros(len(verts_pos), ag._abi.VERTEX_DTYPE)
    verts["pos"] = verts_pos.astype(np.float32)
    b.add_mesh("mesh", verts, faces.astype(np.uint32))
    b.add_instance("mesh", m)
    return b, verts["pos"].astype(np.float64)


def test_closed_icosphere_from_inside():
    v, f = scenes.icosphere(3)
    b, p = _scene(v, f)
    sc = oracle_py.OracleScene(b.desc())
    try:
        targets = np.concatenate([p, 0.5 * (p[f[:, 0]] + p[f[:, 1]]), 0.5 * (p[f[:, 1]] + p[f[:, 2]])])
        rng = np.random.default_rng(3)
        origins = rng.normal(size=targets.shape) * 0.05
        dirs = targets - origins
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        misses = sum(sc.trace(origins[k].astype(np.float32), dirs[k].astype(np.float32), 0.0, 1e10) is None
                     for k in range(len(targets)))
        assert misses == 0
    finally:
        sc.close()


def test_irregular_tiled_plane_at_vertices_and_edges():
    # a 12 x 12 grid of quads, every one split into two triangles along a
    # random diagonal, interior vertices jittered in the plane: rays from
    # above at random slants, aimed at every vertex and every edge midpoint
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
    b, p = _scene(pos, faces)
    sc = oracle_py.OracleScene(b.desc())
    try:
        edges = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        targets = np.concatenate([p[inner], 0.5 * (p[edges[:, 0]] + p[edges[:, 1]])])
        keep = (np.abs(targets[:, 0]) < 0.99) & (np.abs(targets[:, 1]) < 0.99)  # off the outer rim
        targets = targets[keep]
        slant = rng.uniform(-0.6, 0.6, size=(len(targets), 2))
        origins = targets + np.column_stack([slant, np.ones(len(targets))])
        dirs = targets - origins
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        misses = 0
        for k in range(len(targets)):
            r = sc.trace(origins[k].astype(np.float32), dirs[k].astype(np.float32), 0.0, 1e10)
            misses += r is None
        assert misses == 0 and len(targets) > 500
    finally:
        sc.close()
