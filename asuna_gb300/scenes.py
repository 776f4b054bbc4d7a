"""Seeded procedural scenes of the benchmark configurations.

* ``box_scene``   — small closed box (5 quads, 10 triangles, open toward the
  camera), two cuboids rotated +-18 deg about y (24 triangles), Lambertian
  white 0.73 / red (0.65,0.05,0.05) / green (0.12,0.45,0.15), one 0.5 x 0.4
  rectangle light at the ceiling with radiance (17,12,4), pinhole camera at
  z = 3.9 with a 40 deg field of view.
* ``mixed_scene`` — N subdivided icospheres (level 7: 327,680 triangles each)
  displaced by seeded 3-octave value noise (amplitude 0.05), placed uniformly
  in a 20^3 box above a ground quad; materials 40% Lambertian (albedo
  U[0.1,0.9]^3), 40% rough plastic (GGX alpha U[0.05,0.8], ior 1.5), 20%
  dielectric (ior 1.5); a 1024x512 environment map, lognormal(0, 1.5) per
  texel with one 8x8 hotspot x1000; 4 triangle lights; thin-lens camera with
  aperture 0.05.

All data are synthetic (no dataset): shapes and value distributions follow
the configurations, values come from numpy's seeded generator.
"""
import math

import numpy as np

from . import _abi as A
from .scene import SceneBuilder, make_shot, perspective_camera


def _quad(p0, p1, p2, p3, normal):
    v = np.zeros(4, A.VERTEX_DTYPE)
    v["pos"] = [p0, p1, p2, p3]
    v["normal"] = normal
    v["uv"] = [(0, 0), (1, 0), (1, 1), (0, 1)]
    return v, np.array([0, 1, 2, 0, 2, 3], np.uint32)


def cuboid_mesh(hx, hy, hz):
    """Axis-aligned cuboid centred at the origin, 24 vertices (flat faces), 12 triangles."""
    faces = []
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            n = np.zeros(3, np.float32)
            n[axis] = sgn
            u = np.zeros(3, np.float32)
            w = np.zeros(3, np.float32)
            u[(axis + 1) % 3] = 1
            w[(axis + 2) % 3] = 1
            if sgn < 0:
                u, w = w, u
            h = np.array([hx, hy, hz], np.float32)
            c = n * h
            du, dw = u * h, w * h
            faces.append(_quad(c - du - dw, c + du - dw, c + du + dw, c - du + dw, n))
    verts = np.concatenate([f[0] for f in faces])
    idx = np.concatenate([f[1] + 4 * k for k, f in enumerate(faces)]).astype(np.uint32)
    return verts, idx


def rot_y(deg, t):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s, t[0]], [0, 1, 0, t[1]], [-s, 0, c, t[2]]], np.float32)


def box_scene(width=256, height=256, frames=16, max_depth=8, channels=("albedo", "normal", "depth"), seed=0):
    """The small box scene; returns (builder, shot)."""
    b = SceneBuilder()
    white = b.add_lambertian("white", (0.73, 0.73, 0.73))
    red = b.add_lambertian("red", (0.65, 0.05, 0.05))
    green = b.add_lambertian("green", (0.12, 0.45, 0.15))
    # the light is added first, as the reference's loader parses lights before meshes
    b.add_rect_light((-0.25, 0.999, -0.2), (0.25, 0.999, -0.2), (-0.25, 0.999, 0.2), (17.0, 12.0, 4.0))
    quads = {
        "floor": ([(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)], (0, 1, 0), white),
        "ceiling": ([(-1, 1, 1), (1, 1, 1), (1, 1, -1), (-1, 1, -1)], (0, -1, 0), white),
        "back": ([(-1, -1, -1), (-1, 1, -1), (1, 1, -1), (1, -1, -1)], (0, 0, 1), white),
        "left": ([(-1, -1, 1), (-1, 1, 1), (-1, 1, -1), (-1, -1, -1)], (1, 0, 0), red),
        "right": ([(1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)], (-1, 0, 0), green),
    }
    for name, (pts, n, mat) in quads.items():
        v, i = _quad(*[np.array(p, np.float32) for p in pts], np.array(n, np.float32))
        b.add_mesh(name, v, i)
        b.add_instance(name, mat)
    v, i = cuboid_mesh(0.3, 0.3, 0.3)
    b.add_mesh("short_box", v, i)
    b.add_instance("short_box", white, rot_y(-18.0, (0.35, -0.7, 0.35)))
    v, i = cuboid_mesh(0.3, 0.6, 0.3)
    b.add_mesh("tall_box", v, i)
    b.add_instance("tall_box", white, rot_y(18.0, (-0.35, -0.4, -0.35)))
    state, depth = b.state(spp=frames, max_path_depth=max_depth, channels=channels)
    cam = perspective_camera((0, 0, 3.9), (0, 0, 0), (0, 1, 0), 40.0, width, height)
    return b, make_shot(cam, state, width, height, frames, seed=seed, depth_channel=depth)


# ---- icospheres + value noise ---------------------------------------------------
def icosphere(level):
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    for _ in range(level):
        a, b_, c = f[:, 0], f[:, 1], f[:, 2]
        e = np.concatenate([np.stack([a, b_], 1), np.stack([b_, c], 1), np.stack([c, a], 1)])
        lo, hi = e.min(1), e.max(1)
        key = lo * len(v) + hi
        uk, inv = np.unique(key, return_inverse=True)
        mid = v[uk // len(v)] + v[uk % len(v)]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        m = inv.reshape(3, -1) + base
        ab, bc, ca = m[0], m[1], m[2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b_, bc, ab], 1), np.stack([c, ca, bc], 1),
                            np.stack([ab, bc, ca], 1)])
    return v, f


def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint32) * np.uint32(73856093)) ^ (iy.astype(np.uint32) * np.uint32(19349663)) ^ \
        (iz.astype(np.uint32) * np.uint32(83492791)) ^ np.uint32(seed)
    h ^= h >> np.uint32(16)
    h *= np.uint32(0x7FEB352D)
    h ^= h >> np.uint32(15)
    h *= np.uint32(0x846CA68B)
    h ^= h >> np.uint32(16)
    return h.astype(np.float64) * (2.0 / 4294967295.0) - 1.0


def value_noise(p, seed):
    """3D value noise in [-1, 1]: hashed lattice values, smoothstep-trilinear."""
    fl = np.floor(p)
    i = fl.astype(np.int64)
    t = p - fl
    w = t * t * (3.0 - 2.0 * t)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                val = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
                wx = w[:, 0] if dx else 1 - w[:, 0]
                wy = w[:, 1] if dy else 1 - w[:, 1]
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out += val * wx * wy * wz
    return out


def displaced_sphere(base_v, faces, seed, amplitude=0.05, octaves=3, freq=2.0):
    n = np.zeros(len(base_v))
    amp, norm = 1.0, 0.0
    for o in range(octaves):
        n += amp * value_noise(base_v * (freq * 2 ** o) + 17.0 * o, seed * 7919 + o)
        norm += amp
        amp *= 0.5
    pos = base_v * (1.0 + amplitude * n / norm)[:, None]
    # area-weighted vertex normals of the displaced surface
    e1 = pos[faces[:, 1]] - pos[faces[:, 0]]
    e2 = pos[faces[:, 2]] - pos[faces[:, 0]]
    fn = np.cross(e1, e2)
    vn = np.zeros_like(pos)
    for k in range(3):
        for c in range(3):
            vn[:, c] += np.bincount(faces[:, k], weights=fn[:, c], minlength=len(pos))
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)
    v = np.zeros(len(pos), A.VERTEX_DTYPE)
    v["pos"] = pos.astype(np.float32)
    v["normal"] = vn.astype(np.float32)
    return v


def lognormal_envmap(rng, width=1024, height=512, hotspot=8, boost=1000.0):
    env = rng.lognormal(0.0, 1.5, size=(height, width, 3)).astype(np.float32)
    y = int(rng.integers(height // 8, height // 3))
    x = int(rng.integers(0, width - hotspot))
    env[y:y + hotspot, x:x + hotspot] *= np.float32(boost)
    return env


def mixed_scene(width=1920, height=1080, frames=64, max_depth=12, n_spheres=64, level=7, seed=1234,
                rr_depth=3, env_size=(1024, 512), channels=("albedo", "normal", "depth"), verbose=False,
                eye=(0.0, 4.0, 30.0), at=(0.0, -2.0, 0.0)):
    """The mid-size mixed-material scene; returns (builder, shot)."""
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    # lights first (the reference's loader order): 4 triangle lights above the spheres
    for k in range(4):
        cx, cz = -6.0 + 4.0 * k, float(rng.uniform(-6, 6))
        y = 14.0
        b.add_triangle_light((cx - 1.2, y, cz - 1.0), (cx, y, cz + 1.4), (cx + 1.2, y, cz - 1.0), (40.0, 38.0, 34.0))
    b.set_envmap(lognormal_envmap(rng, env_size[0], env_size[1]))
    ground = b.add_lambertian("ground", (0.5, 0.5, 0.5))
    v, i = _quad(np.array((-40, -11, 40), np.float32), np.array((40, -11, 40), np.float32),
                 np.array((40, -11, -40), np.float32), np.array((-40, -11, -40), np.float32),
                 np.array((0, 1, 0), np.float32))
    b.add_mesh("ground", v, i)
    b.add_instance("ground", ground)
    base_v, faces = icosphere(level)
    idx = faces.astype(np.uint32).reshape(-1)
    for k in range(n_spheres):
        u = rng.random()
        if u < 0.4:
            mat = b.add_lambertian(f"m{k}", rng.uniform(0.1, 0.9, 3))
        elif u < 0.8:
            a = float(rng.uniform(0.05, 0.8))
            mat = b.add_rough_plastic(f"m{k}", rng.uniform(0.1, 0.9, 3), (a, a), 1.5)
        else:
            mat = b.add_dielectric(f"m{k}", 1.5)
        pos = rng.uniform(-10.0, 10.0, 3)
        b.add_mesh(f"sphere{k}", displaced_sphere(base_v, faces, seed + 31 * k), idx)
        b.add_instance(f"sphere{k}", mat, np.array([[1, 0, 0, pos[0]], [0, 1, 0, pos[1]], [0, 0, 1, pos[2]]],
                                                   np.float32))
        if verbose and k % 16 == 15:
            print(f"mixed_scene: {k + 1}/{n_spheres} spheres", flush=True)
    return b, mixed_shot(b, width, height, frames, max_depth, rr_depth, channels, eye, at)


def mixed_shot(b, width, height, frames, max_depth=12, rr_depth=3, channels=("albedo", "normal", "depth"),
               eye=(0.0, 4.0, 30.0), at=(0.0, -2.0, 0.0), seed=0):
    """A shot of a mixed-recipe scene `b` (thin lens focused on `at`) at any
    resolution and sample count, without rebuilding the geometry."""
    state, depth = b.state(spp=frames, max_path_depth=max_depth, channels=channels)
    eye, at = np.asarray(eye, np.float64), np.asarray(at, np.float64)
    cam = perspective_camera(eye, at, (0, 1, 0), 50.0, width, height, aperture=0.05,
                             focal_distance=float(np.linalg.norm(eye - at)))
    return make_shot(cam, state, width, height, frames, seed=seed, depth_channel=depth, rr_depth=rr_depth)


def furnace_scene(albedo=(1.0, 1.0, 1.0), width=24, height=24, frames=32, max_depth=8, background=(1.0, 1.0, 1.0)):
    """A flat-shaded convex polyhedron (level-2 icosphere, use_face_normal)
    of Lambertian `albedo` under a uniform background and no lights: every
    camera ray that hits it converges to albedo x background (a white one
    disappears), every other to the background.  Returns (builder, shot,
    mask of the pixels whose samples all see the object, mask of those whose
    samples all miss it)."""
    b = SceneBuilder()
    m = b.add_lambertian("grey", albedo)
    vtx, faces = icosphere(2)
    v = np.zeros(len(vtx), A.VERTEX_DTYPE)
    v["pos"] = vtx
    v["normal"] = vtx
    b.add_mesh("ball", v, faces.astype(np.uint32).reshape(-1))
    b.add_instance("ball", m)
    state, depth = b.state(spp=frames, max_path_depth=max_depth, channels=(), bg_color=background)
    state.use_face_normal = 1
    eye, at = (0.0, 0.0, 3.2), (0.0, 0.0, 0.0)
    cam = perspective_camera(eye, at, (0, 1, 0), 45.0, width, height)
    shot = make_shot(cam, state, width, height, frames, seed=0, depth_channel=depth)
    # pixel centres inside the object's silhouette (the inscribed radius of
    # the polyhedron, in the image plane of a 45-degree horizontal fov)
    ys, xs = np.mgrid[0:height, 0:width]
    px = (xs + 0.5) / width * 2 - 1
    py = ((ys + 0.5) / height * 2 - 1) * height / width
    tan = math.tan(math.radians(45.0) / 2)
    ang = np.arctan(np.hypot(px, py) * tan)
    inside = np.sin(ang) * 3.2 < 0.9  # inscribed radius 0.98, less a pixel footprint
    outside = np.sin(ang) * 3.2 > 1.1  # circumscribed radius 1, plus a pixel footprint
    return b, shot, inside, outside


def _spherical_uv(v):
    """u = longitude, v = colatitude of each vertex (in place)."""
    p = v["pos"].astype(np.float64)
    r = np.maximum(np.linalg.norm(p, axis=1), 1e-12)
    v["uv"][:, 0] = np.arctan2(p[:, 2], p[:, 0]) / (2 * np.pi) + 0.5
    v["uv"][:, 1] = np.arccos(np.clip(p[:, 1] / r, -1, 1)) / np.pi
    return v


def _plugin_textures(b, rng):
    """Procedural textures for every slot a material shader reads; returns
    their ids by role."""
    yy, xx = np.mgrid[0:32, 0:64].astype(np.float32)
    chk = ((xx // 8 + yy // 8) % 2)[..., None]
    smooth = 0.5 + 0.5 * np.sin(xx / 5.0)[..., None] * np.cos(yy / 3.0)[..., None]
    diffuse = (chk * np.array([0.8, 0.55, 0.2]) + (1 - chk) * np.array([0.15, 0.35, 0.7])) * (0.6 + 0.4 * smooth)
    bump = np.stack([0.35 * np.sin(xx / 3.0), 0.35 * np.cos(yy / 2.5), np.ones_like(xx)], -1)
    bump /= np.linalg.norm(bump, axis=-1, keepdims=True)
    obj_n = np.stack([np.sin(xx / 10.0), np.cos(yy / 6.0), 0.5 + 0.5 * np.sin(xx / 4.0)], -1)
    obj_n /= np.linalg.norm(obj_n, axis=-1, keepdims=True)
    tangent = np.stack([np.cos(xx / 9.0), 0.3 * np.sin(yy / 4.0), np.sin(xx / 9.0)], -1)
    tangent /= np.linalg.norm(tangent, axis=-1, keepdims=True)
    alpha = np.stack([0.05 + 0.5 * smooth[..., 0], 0.05 + 0.4 * chk[..., 0], np.zeros_like(xx)], -1)
    metal = np.stack([smooth[..., 0], 0.2 + 0.6 * chk[..., 0], 0.3 + 0.2 * smooth[..., 0]], -1)
    glow = np.stack([2.0 + 2.0 * smooth[..., 0], 1.0 + chk[..., 0], 0.5 * np.ones_like(xx)], -1)
    noise = rng.uniform(0.0, 0.05, (32, 64, 3))
    return {"diffuse": b.add_texture("checker", diffuse + noise), "normal": b.add_texture("bumps", 0.5 * bump + 0.5),
            "object_normal": b.add_texture("object_normals", 0.5 * obj_n + 0.5),
            "tangent": b.add_texture("tangents", 0.5 * tangent + 0.5), "alpha": b.add_texture("alpha", alpha),
            "metal": b.add_texture("metal", metal), "glow": b.add_texture("glow", glow)}


def plugin_scene(width=48, height=32, frames=3, max_depth=8, env=True, opencv=False, seed=11,
                 channels=("albedo", "normal", "depth", "position", "uv", "tangent", "roughness"), textured=False,
                 opacity=False):
    """Every implemented plugin in one small scene: Lambertian, anisotropic
    rough plastic, dielectric, smooth plastic, mirror, conductor, rough
    conductor, Phong, PBR metalness-roughness, Disney (every lobe on) and
    kang18 spheres and an emissive cuboid on a ground quad; a single-sided rect
    light, a double-sided JSON "triangle" light (rect with half area), a mesh
    triangle light, a point light and a distant light; an optional lognormal
    environment map (else a background colour); a thin-lens perspective or an
    OpenCV pinhole camera.  `textured`: spherical UVs on the spheres and a
    texture in every slot the shaders read (diffuse, alpha, metalness and
    roughness, specular, tangent-space and object-space normal maps, tangent
    map, emissive radiance).  `opacity`: the PBR, Disney and kang18 spheres
    let rays pass through (opacity 0.35 / 0.5 / 0.3; Disney's from a mask
    texture when `textured`)."""
    rng = np.random.default_rng(seed)
    b = SceneBuilder()
    b.add_rect_light((-1.0, 3.0, -1.0), (0.0, 3.0, -1.0), (-1.0, 3.0, 0.0), (6.0, 5.0, 4.0))
    b.add_rect_light((1.5, 2.0, -2.0), (2.5, 2.0, -2.0), (1.5, 3.0, -2.0), (3.0, 3.0, 5.0), double_side=True,
                     triangle=True)
    b.add_triangle_light((-2.5, 2.5, 0.5), (-1.5, 2.5, 0.5), (-2.0, 2.5, -0.5), (8.0, 8.0, 8.0))
    b.add_point_light((0.5, 2.0, 1.5), (4.0, 4.0, 4.0))
    b.add_distant_light((0.3, -1.0, -0.2), (0.8, 0.7, 0.6))
    if env:
        b.set_envmap(lognormal_envmap(rng, 32, 16, hotspot=2, boost=50.0))
    g = b.add_lambertian("ground", (0.6, 0.6, 0.55))
    lam = b.add_lambertian("lam", (0.8, 0.3, 0.2))
    rp = b.add_rough_plastic("plastic", (0.2, 0.4, 0.8), (0.2, 0.5), 1.5)
    di = b.add_dielectric("glass", 1.5)
    em = b.add_emissive("lamp", (3.0, 1.5, 0.5))
    sp = b.add_plastic("smooth_plastic", (0.7, 0.65, 0.1), 1.6)
    mi = b.add_mirror("mirror", (0.9, 0.9, 0.95))
    au = b.add_conductor("gold", "Au", (1.0, 1.0, 1.0))
    al = b.add_conductor("rough_aluminium", "Al", (0.9, 0.9, 0.9), alpha=(0.15, 0.3))
    ph = b.add_phong("phong", (0.3, 0.5, 0.2), (0.5, 0.5, 0.45), 40.0)
    pb = b.add_pbr("pbr_metal", (0.9, 0.6, 0.3), metalness=0.7, roughness=0.35)
    dn = b.add_disney("disney", (0.25, 0.45, 0.85), metallic=0.3, roughness=0.4, subsurface=0.5, specular_tint=0.3,
                      sheen=0.6, sheen_tint=0.5, clearcoat=0.8, clearcoat_gloss=0.7, anisotropic=0.5)
    kg = b.add_kang18("kang18", (0.5, 0.3, 0.3), (0.4, 0.4, 0.5), (0.1, 0.3))
    if textured:
        tx = _plugin_textures(b, rng)
        M = b.materials
        M[g].diffuse_texture_id = tx["diffuse"]
        M[lam].diffuse_texture_id, M[lam].normal_texture_id = tx["diffuse"], tx["normal"]
        M[rp].diffuse_texture_id, M[rp].roughness_texture_id, M[rp].normal_texture_id = (tx["diffuse"], tx["alpha"],
                                                                                         tx["normal"])
        M[di].normal_texture_id = tx["normal"]
        M[em].radiance_texture_id = tx["glow"]
        M[sp].normal_texture_id = tx["normal"]
        M[mi].diffuse_texture_id = tx["diffuse"]
        M[au].normal_texture_id = tx["normal"]
        M[al].roughness_texture_id = tx["alpha"]
        M[ph].diffuse_texture_id, M[ph].normal_texture_id = tx["diffuse"], tx["normal"]
        M[pb].metalness_texture_id, M[pb].roughness_texture_id, M[pb].normal_texture_id = (tx["metal"], tx["alpha"],
                                                                                           tx["normal"])
        M[dn].metalness_texture_id, M[dn].roughness_texture_id, M[dn].diffuse_texture_id = (tx["metal"], tx["alpha"],
                                                                                            tx["diffuse"])
        M[kg].metalness_texture_id, M[kg].roughness_texture_id = tx["metal"], tx["alpha"]
        M[kg].normal_texture_id, M[kg].tangent_texture_id = tx["object_normal"], tx["tangent"]
    if opacity:
        b.materials[pb].specular = 0.35
        b.materials[dn].rho_spec[0] = 0.5
        b.materials[kg].metalness = 0.3
        if textured:
            yy, xx = np.mgrid[0:16, 0:32]
            mask = np.repeat(((xx // 4 + yy // 4) % 2).astype(np.float32)[..., None], 3, 2) * 0.9
            b.materials[dn].opacity_texture_id = b.add_texture("mask", mask)
    v, i = cuboid_mesh(0.15, 0.15, 0.15)
    b.add_mesh("lamp", v, i)
    b.add_instance("lamp", em, rot_y(30.0, (0.6, -0.85, 1.2)))
    v, i = _quad(np.array((-4, -1, 4), np.float32), np.array((4, -1, 4), np.float32),
                 np.array((4, -1, -4), np.float32), np.array((-4, -1, -4), np.float32),
                 np.array((0, 1, 0), np.float32))
    b.add_mesh("ground", v, i)
    b.add_instance("ground", g)
    base_v, faces = icosphere(3)
    idx = faces.astype(np.uint32).reshape(-1)
    spheres = [(lam, (-1.3, -0.2, 0.0), 0.8), (rp, (0.0, -0.1, -0.6), 0.8), (di, (1.2, -0.2, 0.3), 0.8),
               (sp, (-0.4, -0.6, 1.1), 0.4), (mi, (0.75, -0.62, 1.3), 0.38), (au, (-1.6, -0.65, 1.4), 0.35),
               (al, (1.75, -0.6, 1.2), 0.4), (ph, (0.2, -0.7, 2.0), 0.3), (pb, (-0.9, -0.72, 2.1), 0.28),
               (dn, (1.0, -0.7, 2.2), 0.3), (kg, (-0.3, -0.75, 2.6), 0.25)]
    for k, (mat, pos, s) in enumerate(spheres):
        sv = displaced_sphere(base_v, faces, seed + k, amplitude=0.05)
        b.add_mesh(f"s{k}", _spherical_uv(sv) if textured else sv, idx)
        b.add_instance(f"s{k}", mat, np.array([[s, 0, 0, pos[0]], [0, s, 0, pos[1]], [0, 0, s, pos[2]]], np.float32))
    state, depth = b.state(spp=frames, max_path_depth=max_depth, channels=channels, bg_color=(0.2, 0.25, 0.3))
    eye, at = (0.0, 1.0, 5.0), (0.0, -0.3, 0.0)
    if opencv:
        from .scene import opencv_camera
        cam = opencv_camera(eye, at, (0, 1, 0), (0.9 * width, 0.9 * width, 0.5 * width, 0.5 * height))
    else:
        cam = perspective_camera(eye, at, (0, 1, 0), 55.0, width, height, aperture=0.05, focal_distance=5.0)
    return b, make_shot(cam, state, width, height, frames, seed=0, depth_channel=depth)


def training_scene(seed, width=128, height=128, frames=4, max_depth=8, level=4):
    """A scene of the mixed-scene recipe with a seeded sphere count (4..24)
    and a seeded camera on a ring around the spheres: the denoiser's
    training and evaluation scenes.  Returns (builder, shot)."""
    rng = np.random.default_rng(10_000 + seed)
    n = int(rng.integers(4, 25))
    ang = float(rng.uniform(0.0, 2.0 * np.pi))
    r = float(rng.uniform(16.0, 30.0))
    eye = (r * np.sin(ang), float(rng.uniform(-4.0, 12.0)), r * np.cos(ang))
    at = tuple(float(v) for v in rng.uniform(-4.0, 4.0, 3))
    return mixed_scene(width, height, frames=frames, max_depth=max_depth, n_spheres=n, level=level, seed=seed,
                       rr_depth=3, env_size=(128, 64), eye=eye, at=at)


def stacked_instances_scene(n_instances, width=8, height=8):
    """n copies of one triangle at the same place, facing the camera, lit by
    a point light: every camera ray meets every copy at the same distance, so
    its traversal enters and leaves all n instances.  For n in the tens of
    thousands that passes the traversal's loop bound (65,536 leaves and
    transitions per ray): a scene for the error path of a runaway traversal."""
    b = SceneBuilder()
    white = b.add_lambertian("white", (0.73, 0.73, 0.73))
    b.add_point_light((0.0, 0.0, 2.0), (1.0, 1.0, 1.0))
    v = np.zeros(3, A.VERTEX_DTYPE)
    v["pos"] = [(-1, -1, 0), (1, -1, 0), (0, 1, 0)]
    v["normal"] = (0, 0, 1)
    b.add_mesh("tri", v, np.array([0, 1, 2], np.uint32))
    for _ in range(n_instances):
        b.add_instance("tri", white)
    state, depth = b.state(spp=1, max_path_depth=1, channels=())
    cam = perspective_camera((0, 0, 3.0), (0, 0, 0), (0, 1, 0), 10.0, width, height)
    return b, make_shot(cam, state, width, height, 1, depth_channel=depth)


def sky_scene(width=48, height=32, frames=3, max_depth=6, dusk=False, point_light=False,
              channels=("albedo", "normal", "depth")):
    """Three level-3 icospheres (Lambertian, rough plastic, dielectric) over a
    small ground quad under the sun & sky environment (GpuSunAndSky in use,
    no environment map).  Day: the reference's default sky, the camera
    pitched up toward the sun so the sun disk and glow are in view; dusk: the
    sun 3 degrees below the horizon (night factor), haze 4, red/blue shift
    0.2, saturation 0.6, a raised horizon, blur 0.5, no physical sun scaling
    and a level camera, half of whose rays miss below the horizon (ground
    colour branch).  With `point_light` a point light shares the light
    sample with the sky."""
    b = SceneBuilder()
    if point_light:
        b.add_point_light((1.5, 3.0, 1.0), (6.0, 5.0, 4.0))
    if dusk:
        a = math.radians(-3.0)
        b.set_sun_and_sky(sun_direction=(0.6 * math.cos(a), math.sin(a), 0.8 * math.cos(a)), haze=4.0,
                          redblueshift=0.2, saturation=0.6, horizon_height=0.5, horizon_blur=0.5,
                          physically_scaled_sun=0, multiplier=2e-5)
    else:
        b.set_sun_and_sky()
    ground = b.add_lambertian("ground", (0.4, 0.4, 0.4))
    v, i = _quad(np.array((-2, -1, 2), np.float32), np.array((2, -1, 2), np.float32),
                 np.array((2, -1, -2), np.float32), np.array((-2, -1, -2), np.float32), np.array((0, 1, 0), np.float32))
    b.add_mesh("ground", v, i)
    b.add_instance("ground", ground)
    base_v, faces = icosphere(3)
    idx = faces.astype(np.uint32).reshape(-1)
    mats = [b.add_lambertian("lam", (0.7, 0.6, 0.5)), b.add_rough_plastic("plastic", (0.2, 0.4, 0.8), (0.2, 0.2)),
            b.add_dielectric("glass", 1.5)]
    for k, (mat, pos) in enumerate(zip(mats, [(-1.3, 0.0, 0.0), (0.0, 0.2, 0.6), (1.3, 0.0, 0.0)])):
        verts = np.zeros(len(base_v), A.VERTEX_DTYPE)
        verts["pos"] = base_v * 0.6
        verts["normal"] = base_v
        b.add_mesh(f"s{k}", verts, idx)
        b.add_instance(f"s{k}", mat, np.array([[1, 0, 0, pos[0]], [0, 1, 0, pos[1]], [0, 0, 1, pos[2]]], np.float32))
    state, depth = b.state(spp=frames, max_path_depth=max_depth, channels=channels)
    eye, at = ((0.0, 0.3, -5.0), (0.0, 0.3, 0.0)) if dusk else ((0.0, 0.0, -5.0), (0.0, 4.5, 3.0))
    cam = perspective_camera(eye, at, (0, 1, 0), 70.0, width, height)
    return b, make_shot(cam, state, width, height, frames, depth_channel=depth)
