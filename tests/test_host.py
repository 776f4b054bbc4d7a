"""Host side, no GPU: the C ABI library loads and exports every declared
symbol; the JSON scene loader, camera matrices, env tables and fdrInt follow
the reference's host code; errors are reported, never fatal."""
import ctypes as C
import json
import math
import os
import re

import numpy as np
import pytest

import asuna_gb300 as ag
from asuna_gb300 import _abi as A
from asuna_gb300 import scenes
from oracle import oracle_py

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    declared = set()
    for name in sorted(os.listdir(os.path.join(ROOT, "include"))):
        text = open(os.path.join(ROOT, "include", name)).read()
        declared |= set(re.findall(r"^\s*(?:int|float|uint64_t|void\*|void|const char\*)\s+(asuna_\w+)\s*\(", text,
                                   re.M))
    assert len(declared) >= 60
    assert "asuna_denoise" in declared and "asuna_server_submit" in declared
    L = C.CDLL(A.LIB_PATH)
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing
    assert {name for name, _, _ in A.SIGNATURES} <= declared


def test_struct_layouts_match_reference_abi():
    # src/shared/: GpuVertex 44, GpuMaterial 132, GpuLight 76, GpuCamera 224 (std140),
    # GpuPushConstantRaytrace 84
    assert A.VERTEX_DTYPE.itemsize == 44
    assert C.sizeof(A.Material) == 132 and C.sizeof(A.Light) == 76
    assert C.sizeof(A.Camera) == 224 and C.sizeof(A.RtState) == 84
    assert A.Camera.type.offset == 208 and A.RtState.bg_color.offset == 16
    assert A.RtState.env_map_resolution.offset == 40 and A.RtState.uv_out_channel.offset == 80


def test_no_cuda_device_is_an_error_not_a_fallback():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(ag.AsunaError) as e:
        ag.Context(0)
    assert e.value.code == A.ERR_NO_DEVICE


def _np_camera(eye, at, up, fov, w, h):
    """numpy restatement of src/core/camera.cpp:28-99 and camera.h:124-126."""
    eye, at, up = (np.asarray(x, np.float64) for x in (eye, at, up))
    z = eye - at
    z /= np.linalg.norm(z)
    x = np.cross(up, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = x, y, z
    view[:3, 3] = -view[:3, :3] @ eye
    view = np.diag([1.0, -1.0, -1.0, 1.0]) @ view
    c2w = np.linalg.inv(view)
    ctot = 1.0 / math.tan(math.radians(fov) * 0.5)
    n, f = 0.1, 100.0
    persp = np.array([[ctot, 0, 0, 0], [0, ctot, 0, 0], [0, 0, f / (f - n), -n * f / (f - n)], [0, 0, 1, 0]])
    c2r = np.diag([w, h, 1, 1]) @ np.diag([0.5, 0.5, 1, 1]) @ np.array(
        [[1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 0], [0, 0, 0, 1]]) @ np.diag([1, w / h, 1, 1]) @ persp
    return c2w, np.linalg.inv(c2r)


def test_perspective_camera_matrices():
    cam = ag.perspective_camera((0.3, 1.0, 3.9), (0.0, -0.2, 0.1), (0, 1, 0), 40.0, 320, 200)
    c2w, r2c = _np_camera((0.3, 1.0, 3.9), (0.0, -0.2, 0.1), (0, 1, 0), 40.0, 320, 200)
    got_c2w = np.array(cam.camera_to_world).reshape(4, 4).T  # column-major
    got_r2c = np.array(cam.raster_to_camera).reshape(4, 4).T
    assert np.allclose(got_c2w, c2w, atol=1e-6)
    assert np.allclose(got_r2c, r2c, rtol=1e-5, atol=1e-6)
    # the pixel-centre ray of the image centre looks at the target; fov is horizontal
    p = got_r2c @ np.array([160.0, 100.0, 0.0, 1.0])
    d = got_c2w[:3, :3] @ (p[:3] / p[3])
    d /= np.linalg.norm(d)
    t = np.array([0.0, -0.2, 0.1]) - np.array([0.3, 1.0, 3.9])
    assert np.allclose(d, t / np.linalg.norm(t), atol=1e-5)
    pl = got_r2c @ np.array([0.0, 100.0, 0.0, 1.0])
    pr = got_r2c @ np.array([320.0, 100.0, 0.0, 1.0])
    a = np.arctan2(np.abs(pl[0] / pl[3]), pl[2] / pl[3]) + np.arctan2(np.abs(pr[0] / pr[3]), pr[2] / pr[3])
    assert abs(math.degrees(a) - 40.0) < 1e-3


def _np_env_tables(env):
    """numpy restatement of EnvMap::EnvMap (src/core/texture.cpp:144-226)."""
    h, w = env.shape[:2]
    e = env.astype(np.float64)
    weight = (0.3 * e[..., 0] + 0.6 * e[..., 1] + 0.1 * e[..., 2]).astype(np.float32)
    pdf2, cdf2 = np.zeros((h, w), np.float32), np.zeros((h, w), np.float32)
    pdf1, cdf1 = np.zeros(h, np.float32), np.zeros(h, np.float32)
    total = np.float32(0)
    for j in range(h):
        acc = np.float32(0)
        for i in range(w):
            acc = np.float32(acc + weight[j, i])
            cdf2[j, i] = acc
        pdf2[j] = (weight[j].astype(np.float64) / (np.float64(acc) + 1e-7)).astype(np.float32)
        cdf2[j] = (cdf2[j].astype(np.float64) / (np.float64(acc) + 1e-7)).astype(np.float32)
        total = np.float32(total + acc)
        pdf1[j], cdf1[j] = acc, total
    cdf1 = (cdf1.astype(np.float64) / (np.float64(total) + 1e-7)).astype(np.float32)
    pdf1 = (pdf1.astype(np.float64) / (np.float64(total) + 1e-7)).astype(np.float32)
    marg, cond = np.zeros((h, w, 2), np.float32), np.zeros((h, w, 2), np.float32)
    for j in range(h):
        marg[j, 0] = (np.float32(np.searchsorted(cdf1, np.float32(j + 1) / np.float32(h), "left")) / np.float32(h),
                      pdf1[j])
        cols = np.searchsorted(cdf2[j], (np.arange(1, w + 1, dtype=np.float32) / np.float32(w)), "left")
        cond[j, :, 0] = cols.astype(np.float32) / np.float32(w)
        cond[j, :, 1] = pdf2[j]
    return marg, cond


def test_envmap_tables():
    rng = np.random.default_rng(3)
    env = scenes.lognormal_envmap(rng, 24, 12, hotspot=2, boost=100.0)
    rgba = np.concatenate([env, np.ones(env.shape[:2] + (1,), np.float32)], 2)
    marg, cond = ag.envmap_tables(rgba)
    nm, nc = _np_env_tables(rgba)
    assert np.array_equal(marg, nm) and np.array_equal(cond, nc)
    om, oc = np.zeros_like(marg), np.zeros_like(cond)
    L = oracle_py.port()
    rgba = np.ascontiguousarray(rgba)
    assert L.oracle_envmap_tables(24, 12, rgba.ctypes.data, om.ctypes.data, oc.ctypes.data) == 0
    assert np.array_equal(marg, om) and np.array_equal(cond, oc)


def _np_fdr(ior, n):
    """numpy restatement of computeDiffuseFresnel (src/loader/material.cpp:6-37)."""
    def refl(eta, c):
        eta, c = np.float32(eta), np.float32(c)
        if c < 0:
            eta, c = np.float32(1) / eta, -c
        s2 = eta * eta * (np.float32(1) - c * c)
        if s2 > 1:
            return np.float32(1)
        ct = np.sqrt(max(np.float32(1) - s2, np.float32(0)))
        rs = (eta * c - ct) / (eta * c + ct)
        rp = (eta * ct - c) / (eta * ct + c)
        return (rs * rs + rp * rp) * np.float32(0.5)
    acc = 0.0
    fb = refl(ior, 0.0)
    for i in range(1, n + 1):
        fa = refl(ior, min(np.sqrt(np.float32(i) / np.float32(n)), np.float32(1)))
        acc += float(np.float32(fa + fb)) * (0.5 / n)
        fb = fa
    return np.float32(acc)


@pytest.mark.parametrize("ior", [1.33, 1.5, 2.4])
def test_diffuse_fresnel(ior):
    assert A.lib().asuna_diffuse_fresnel(C.c_float(ior), 1000) == pytest.approx(float(_np_fdr(ior, 1000)), abs=0)


def _write_box_json(tmp, frames=4):
    """The box scene as an Asuna scene file + OBJ meshes."""
    def obj(path, verts, idx, normals):
        with open(path, "w") as f:
            for v in verts:
                f.write("v %r %r %r\n" % tuple(float(x) for x in v))
            for n in normals:
                f.write("vn %r %r %r\n" % tuple(float(x) for x in n))
            for t in range(0, len(idx), 3):
                a, b, c = idx[t:t + 3] + 1
                f.write(f"f {a}//{a} {b}//{b} {c}//{c}\n")
    b, shot = scenes.box_scene(32, 32, frames=frames, max_depth=6, channels=("albedo", "normal", "depth"))
    meshes, instances = [], []
    for k, (name, (v, i)) in enumerate(zip(b.mesh_names, b.meshes)):
        if name.startswith("__"):
            continue
        obj(os.path.join(tmp, name + ".obj"), v["pos"], i, v["normal"])
        meshes.append({"name": name, "path": name + ".obj"})
    for t, m, mat, light in b.instances:
        if light >= 0:
            continue
        inst = {"mesh": b.mesh_names[m], "material": b.material_names[mat]}
        if not np.array_equal(t, np.eye(3, 4, dtype=np.float32)):
            full = np.eye(4)
            full[:3] = t
            inst["toworld"] = [{"type": "matrix", "value": [float(x) for x in full.reshape(-1)]}]
        instances.append(inst)
    scene = {
        "state": {"path_tracing": {"spp": frames, "max_path_depth": 6, "multi_channel": ["albedo", "normal", "depth"]}},
        "camera": {"type": "perspective", "fov": 40.0, "film": {"resolution": [32, 32]}},
        "materials": [{"type": "brdf_lambertian", "name": n, "diffuse_reflectance": list(b.materials[i].diffuse)}
                      for i, n in enumerate(b.material_names) if i > 0],
        "lights": [{"type": "rect", "position": [-0.25, 0.999, -0.2], "v1": [0.25, 0.999, -0.2],
                    "v2": [-0.25, 0.999, 0.2], "radiance": [17, 12, 4]}],
        "meshes": meshes,
        "instances": instances,
        "shots": [{"type": "lookat", "eye": [0, 0, 3.9], "lookat": [0, 0, 0], "up": [0, 1, 0]}],
    }
    path = os.path.join(tmp, "box.json")
    with open(path, "w") as f:
        json.dump(scene, f)
    return path, b, shot


def test_json_loader_matches_builder(tmp_path):
    path, b, shot = _write_box_json(str(tmp_path))
    js = ag.JsonScene(path)
    d = js.desc().desc
    assert d.num_lights == 2 and d.lights[1].type == A.LIGHT_RECT
    assert d.num_materials == len(b.materials) and d.num_instances == len(b.instances)
    for k in range(d.num_materials):
        assert bytes(d.materials[k]) == bytes(b.materials[k])
    assert bytes(d.lights[1]) == bytes(b.lights[1])
    # world-space triangles per instance agree (OBJ meshes are de-indexed)
    for k in range(d.num_instances):
        di = d.instances[k]
        t, m, mat, light = b.instances[k]
        assert di.light_id == light and (light >= 0 or di.material_id == mat)
        md = d.meshes[di.mesh_id]
        v = np.ctypeslib.as_array(C.cast(md.vertices, C.POINTER(C.c_float)), (md.num_vertices * 11,))
        v = v.reshape(-1, 11)
        idx = np.ctypeslib.as_array(C.cast(md.indices, C.POINTER(C.c_uint32)), (md.num_triangles * 3,))
        got = v[idx, 0:3]
        bv, bi = b.meshes[m]
        assert np.array_equal(got, bv["pos"][bi])
        assert np.allclose(np.array(di.transform).reshape(3, 4), t, atol=1e-7)
    shots = js.shots()
    assert len(shots) == 1 and shots[0].frames == 4 and shots[0].state.num_lights == 1
    assert shots[0].depth_out_channel == 2 and shots[0].state.diffuse_out_channel == 0
    assert bytes(shots[0].camera) == bytes(shot.camera)
    assert js.channels() == [A.CH_DIFFUSE, A.CH_NORMAL, A.CH_DEPTH]


def test_json_scene_renders_like_builder_on_oracle(tmp_path):
    path, b, shot = _write_box_json(str(tmp_path), frames=2)
    js = ag.JsonScene(path)
    s = js.shots()[0]
    s.depth_out_channel = shot.depth_out_channel = -1
    f1, r1, _ = oracle_py.OracleScene(js.desc()).render(s)
    f2, r2, _ = oracle_py.OracleScene(b.desc()).render(shot)
    # meshes differ only by OBJ de-indexing; radiance agrees path for path
    assert np.allclose(r1["radiance"], r2["radiance"], rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("text,code", [
    ("{", A.ERR_PARSE),
    ('{"state": {}, "camera": {"type": "perspective", "film": {"resolution": [8, 8]}}, "meshes": []}', A.ERR_PARSE),
    ('{"state": {}, "camera": {"type": "fisheye", "film": {"resolution": [8, 8]}}, "meshes": [], "instances": []}',
     A.ERR_PARSE),
    ('{"state": {}, "camera": {"type": "perspective", "film": {"resolution": [8, 8]}}, "meshes": [], '
     '"instances": [], "materials": [{"type": "brdf_kang18", "name": "d"}]}', A.ERR_PARSE),
    ('{"state": {}, "camera": {"type": "perspective", "film": {"resolution": [8, 8]}}, "meshes": [], '
     '"instances": [], "materials": [{"type": "brdf_velvet", "name": "d"}]}', A.ERR_PARSE),
    ('{"state": {}, "camera": {"type": "perspective", "film": {"resolution": [8, 8]}}, '
     '"meshes": [{"name": "m", "path": "missing.obj"}], "instances": []}', A.ERR_IO),
    ('{"state": {"path_tracing": {"multi_channel": ["a","b","c","d","e","f","g","h"]}}, '
     '"camera": {"type": "perspective", "film": {"resolution": [8, 8]}}, "meshes": [], "instances": []}',
     A.ERR_PARSE),
])
def test_json_errors_are_reported(text, code):
    with pytest.raises(ag.AsunaError) as e:
        ag.JsonScene(text=text, base_dir="/nonexistent")
    assert e.value.code == code
    assert len(str(e.value)) > 20


def test_json_shot_types_and_lights(tmp_path):
    tri = tmp_path / "tri.obj"
    tri.write_text("v 0 2 0\nv 1 2 0\nv 0 2 1\nv 1 2 1\nf 1 2 3\nf 2 4 3\n")
    scene = {
        "state": {"path_tracing": {"spp": 3, "max_path_depth": 5}},
        "camera": {"type": "opencv", "fx": 50, "fy": 50, "cx": 16, "cy": 12, "film": {"resolution": [32, 24]}},
        "lights": [{"type": "triangle", "position": [0, 1, 0], "v1": [1, 1, 0], "v2": [0, 1, 1], "radiance": [1, 1, 1],
                    "double_side": True},
                   {"type": "mesh", "path": "tri.obj", "radiance": [2, 2, 2]},
                   {"type": "point", "position": [0, 3, 0], "radiance": [5, 5, 5]},
                   {"type": "distant", "direction": [0, -1, 0], "radiance": [1, 1, 1]}],
        "meshes": [], "instances": [],
        "shots": [{"type": "toworld", "matrix": [1, 0, 0, 0, 0, 1, 0, 1, 0, 0, 1, -4, 0, 0, 0, 1]},
                  {"type": "opencv", "matrix": [1, 0, 0, 0, 0, -1, 0, 1, 0, 0, -1, 4, 0, 0, 0, 1],
                   "state": {"path_tracing": {"spp": 7}}}],
    }
    js = ag.JsonScene(text=json.dumps(scene), base_dir=str(tmp_path))
    d = js.desc().desc
    # dummy + triangle(-> rect, half area) + 2 mesh facets + point + distant
    assert d.num_lights == 6
    assert d.lights[1].type == A.LIGHT_RECT and d.lights[1].area == pytest.approx(0.5)
    assert d.lights[1].double_side == 1
    assert d.lights[2].type == A.LIGHT_TRIANGLE and d.lights[2].area == pytest.approx(0.5)
    assert d.lights[4].type == A.LIGHT_POINT and d.lights[5].type == A.LIGHT_DIRECTIONAL
    assert d.num_instances == 3  # rect light + two facets
    shots = js.shots()
    assert [s.frames for s in shots] == [3, 7]
    assert shots[0].camera.type == A.CAMERA_OPENCV and shots[0].state.num_lights == 5
    c2w = np.array(shots[0].camera.camera_to_world).reshape(4, 4).T
    assert np.allclose(c2w[:3, 3], [0, 1, -4])


def _read_exr(path):
    """Reader for the uncompressed FLOAT scanline files the library writes."""
    import struct
    data = open(path, "rb").read()
    assert struct.unpack_from("<i", data, 0)[0] == 20000630
    p = 8
    attrs = {}
    while data[p] != 0:
        name_end = data.index(b"\0", p)
        name = data[p:name_end].decode()
        type_end = data.index(b"\0", name_end + 1)
        size = struct.unpack_from("<i", data, type_end + 1)[0]
        attrs[name] = data[type_end + 5:type_end + 5 + size]
        p = type_end + 5 + size
    p += 1
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    assert attrs["compression"] == b"\0"
    offsets = struct.unpack_from(f"<{h}Q", data, p)
    img = np.zeros((h, w, 4), np.float32)
    for y, off in enumerate(offsets):
        yy, size = struct.unpack_from("<ii", data, off)
        ch = np.frombuffer(data, np.float32, 4 * w, off + 8).reshape(4, w)  # A, B, G, R
        img[yy] = ch[::-1].T
    return img


def test_image_writers(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.uniform(-0.5, 4.0, size=(13, 21, 4)).astype(np.float32)
    L = A.lib()
    for ext in ("exr", "png", "pfm"):
        path = str(tmp_path / f"x.{ext}")
        A.check(L.asuna_image_write(path.encode(), 21, 13, img.ctypes.data))
    assert np.array_equal(_read_exr(str(tmp_path / "x.exr")), img)
    import zlib
    data = open(tmp_path / "x.png", "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    idat = data.index(b"IDAT")
    n = int.from_bytes(data[idat - 4:idat], "big")
    raw = np.frombuffer(zlib.decompress(data[idat + 4:idat + 4 + n]), np.uint8).reshape(13, 1 + 21 * 4)
    assert np.all(raw[:, 0] == 0)
    want = (np.clip(img, 0, 1) * 255 + 0.5).astype(np.uint8).reshape(13, -1)
    assert np.array_equal(raw[:, 1:], want)
    w, h = C.c_uint32(), C.c_uint32()
    back = np.zeros((13, 21, 4), np.float32)
    A.check(L.asuna_image_read(str(tmp_path / "x.pfm").encode(), C.byref(w), C.byref(h), back.ctypes.data, back.size))
    assert (w.value, h.value) == (21, 13) and np.array_equal(back[..., :3], img[..., :3])


def test_hdr_envmap_reader(tmp_path):
    # flat (non run-length) Radiance RGBE file
    w, h = 4, 2
    rgbe = np.array([[[128, 64, 32, 129]] * w] * h, np.uint8)
    (tmp_path / "e.hdr").write_bytes(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 2 +X 4\n" + rgbe.tobytes())
    ww, hh = C.c_uint32(), C.c_uint32()
    out = np.zeros((h, w, 4), np.float32)
    A.check(A.lib().asuna_image_read(str(tmp_path / "e.hdr").encode(), C.byref(ww), C.byref(hh), out.ctypes.data,
                                     out.size))
    assert np.allclose(out[..., :3], np.array([128, 64, 32]) * 2.0 ** (129 - 136))


def test_json_textures(tmp_path):
    """"textures" (src/loader/loader.cpp:334-347) load into the scene's
    texture list after the dummy texture; materials reference them by name.
    .hdr / .pfm are read; other image formats are reported as unsupported."""
    rng = np.random.default_rng(2)
    img = rng.uniform(0, 2, (3, 5, 4)).astype(np.float32)
    img[..., 3] = 1.0
    A.check(A.lib().asuna_image_write(str(tmp_path / "t.pfm").encode(), 5, 3, img.ctypes.data))
    base = {"state": {}, "camera": {"type": "perspective", "film": {"resolution": [8, 8]}}, "meshes": [],
            "instances": []}
    scene = {**base, "textures": [{"name": "t", "path": "t.pfm", "gamma": 2.2}],
             "materials": [{"type": "brdf_lambertian", "name": "m", "diffuse_texture": "t", "normal_texture": "t"}]}
    js = ag.JsonScene(text=json.dumps(scene), base_dir=str(tmp_path))
    d = js.desc().desc
    assert d.num_textures == 2 and (d.textures[0].width, d.textures[0].height) == (1, 1)
    t = d.textures[1]
    assert (t.width, t.height) == (5, 3)
    got = np.ctypeslib.as_array(C.cast(t.rgba, C.POINTER(C.c_float)), shape=(3, 5, 4))
    assert np.array_equal(got[..., :3], img[..., :3])
    assert d.materials[1].diffuse_texture_id == 1 and d.materials[1].normal_texture_id == 1
    A.check(A.lib().asuna_scene_validate(js.desc().ptr))
    # a texture id past the list is invalid
    b = ag.SceneBuilder()
    k = b.add_lambertian("m", (0.5, 0.5, 0.5))
    b.materials[k].diffuse_texture_id = 7
    with pytest.raises(ag.AsunaError) as e:
        A.check(A.lib().asuna_scene_validate(b.desc().ptr))
    assert e.value.code == A.ERR_INVALID
    (tmp_path / "p.png").write_bytes(b"not decoded")
    bad = {**base, "textures": [{"name": "p", "path": "p.png"}]}
    with pytest.raises(ag.AsunaError) as e:
        ag.JsonScene(text=json.dumps(bad), base_dir=str(tmp_path))
    assert e.value.code == A.ERR_UNSUPPORTED


def test_json_material_plugins_match_builder():
    """brdf_plastic, brdf_mirror, brdf_conductor, brdf_rough_conductor,
    brdf_phong, brdf_pbr_metalness_roughness, brdf_disney and brdf_kang18
    parse into the same device structs as the builder
    (src/loader/material.cpp:116-143, 156-187, 197-210, 233-243, 306-347,
    359-405); an unknown metal is a parse error."""
    base = {"state": {}, "camera": {"type": "perspective", "film": {"resolution": [8, 8]}}, "meshes": [],
            "instances": []}
    mats = [{"type": "brdf_plastic", "name": "p", "diffuse_reflectance": [0.7, 0.65, 0.1], "ior": 1.6},
            {"type": "brdf_mirror", "name": "m", "diffuse_reflectance": [0.9, 0.9, 0.95]},
            {"type": "brdf_conductor", "name": "au", "material": "Au"},
            {"type": "brdf_rough_conductor", "name": "al", "material": "Al", "diffuse_reflectance": [0.9, 0.9, 0.9],
             "alpha": [0.15, 0.3]},
            {"type": "brdf_conductor", "name": "cu"},
            {"type": "brdf_phong", "name": "ph", "diffuse_reflectance": [0.3, 0.5, 0.2],
             "specular_reflectance": [0.5, 0.5, 0.45], "shininess": 40},
            {"type": "brdf_pbr_metalness_roughness", "name": "pb", "diffuse_reflectance": [0.9, 0.6, 0.3],
             "metalness": 0.7, "roughness": 0.35},
            {"type": "brdf_disney", "name": "dn", "diffuse_reflectance": [0.25, 0.45, 0.85], "metallic": 0.3,
             "roughness": 0.4},
            {"type": "brdf_kang18", "name": "kg", "diffuse_reflectance": [0.5, 0.3, 0.3],
             "specular_reflectance": [0.4, 0.4, 0.5], "alpha": [0.1, 0.3]}]
    js = ag.JsonScene(text=json.dumps({**base, "materials": mats}), base_dir=".")
    d = js.desc().desc
    b = ag.SceneBuilder()
    b.add_plastic("p", (0.7, 0.65, 0.1), 1.6)
    b.add_mirror("m", (0.9, 0.9, 0.95))
    b.add_conductor("au", "Au")
    b.add_conductor("al", "Al", (0.9, 0.9, 0.9), alpha=(0.15, 0.3))
    b.add_conductor("cu")
    b.add_phong("ph", (0.3, 0.5, 0.2), (0.5, 0.5, 0.45), 40.0)
    b.add_pbr("pb", (0.9, 0.6, 0.3), metalness=0.7, roughness=0.35)
    b.add_disney("dn", (0.25, 0.45, 0.85), metallic=0.3, roughness=0.4)
    b.add_kang18("kg", (0.5, 0.3, 0.3), (0.4, 0.4, 0.5), (0.1, 0.3))
    assert d.num_materials == len(b.materials)
    for k in range(1, d.num_materials):
        assert bytes(d.materials[k]) == bytes(b.materials[k]), k
    assert d.materials[1].type == A.MAT_PLASTIC and d.materials[1].radiance[0] == pytest.approx(
        float(_np_fdr(1.6, 1000)), abs=0)
    assert d.materials[3].type == A.MAT_CONDUCTOR and d.materials[4].type == A.MAT_ROUGH_CONDUCTOR
    assert d.materials[6].type == A.MAT_PHONG and d.materials[6].specular == 40.0
    assert list(d.materials[6].rho_spec) == pytest.approx([0.5, 0.5, 0.45])
    # gold: eta (0.1431, 0.3750, 1.4425), k (3.9832, 2.3857, 1.6032)
    assert np.allclose(list(d.materials[3].radiance), [0.1431189557, 0.3749570432, 1.4424785571])
    assert np.allclose(list(d.materials[3].radiance_factor), [3.9831604247, 2.3857207478, 1.6032152899])
    with pytest.raises(ag.AsunaError) as e:
        ag.JsonScene(text=json.dumps({**base, "materials": [{"type": "brdf_conductor", "name": "x",
                                                             "material": "Unobtainium"}]}), base_dir=".")
    assert e.value.code == A.ERR_PARSE
    # Disney's JSON "opacity" lands in rho_spec[0] (pass-through probability)
    js = ag.JsonScene(text=json.dumps({**base, "materials": [{"type": "brdf_disney", "name": "x", "opacity": 0.5}]}),
                      base_dir=".")
    assert js.desc().desc.materials[1].rho_spec[0] == 0.5
    A.check(A.lib().asuna_scene_validate(js.desc().ptr))


def test_post_state_layout_defaults_and_json():
    # GpuPushConstantPost (src/shared/pushconstant.h:50-62): 48 bytes
    assert C.sizeof(A.PostState) == 48
    assert A.PostState.rendering_ratio.offset == 24 and A.PostState.tm_type.offset == 44
    p = ag.default_post()
    assert (p.brightness, p.contrast, p.saturation, p.vignette, p.avg_lum, p.zoom) == (1, 1, 1, 0, 1, 1)
    assert (p.y_white, p.key, p.auto_exposure, p.tm_type) == (0.5, 0.5, 0, A.TONEMAP_FILMIC)
    base = {"camera": {"type": "perspective", "film": {"resolution": [8, 8]}}, "meshes": [], "instances": []}
    for name, t in [("none", 0), ("gamma", 1), ("reinhard", 2), ("Aces", 3), ("filmic", 4), ("pbrt", 5),
                    ("custom", 6)]:
        js = ag.JsonScene(text=json.dumps({**base, "state": {"post_processing": {"tone_mapping": name}}}),
                          base_dir=".")
        q = A.PostState()
        A.check(A.lib().asuna_json_post_state(js.handle, C.byref(q)))
        assert q.tm_type == t


def test_oracle_tonemap_closed_forms():
    L = oracle_py.port()
    rng = np.random.default_rng(4)
    img = rng.gamma(1.0, 0.6, (6, 10, 4)).astype(np.float32)
    out = np.zeros_like(img)

    def run(t):
        p = ag.default_post(t)
        assert L.oracle_tonemap(img.ctypes.data, 10, 6, C.byref(p), out.ctypes.data) == 0
        return out.copy()

    assert np.array_equal(run(A.TONEMAP_NONE), img)
    x = np.maximum(img[..., :3] - np.float32(0.004), np.float32(0))
    hejl = (x * (x * np.float32(6.2) + np.float32(0.5))) / (x * (x * np.float32(6.2) + np.float32(1.7)) + np.float32(0.06))
    assert np.allclose(run(A.TONEMAP_FILMIC)[..., :3], hejl, rtol=1e-6, atol=1e-7)
    c = img[..., :3].astype(np.float64)
    srgb = np.where(c < 0.0031308, 12.92 * c, 1.055 * c ** (1 / 2.4) - 0.055)
    assert np.allclose(run(A.TONEMAP_PBRT)[..., :3], srgb, rtol=1e-5, atol=1e-6)
    assert np.allclose(run(A.TONEMAP_GAMMA)[..., :3], (c / (1 + c / 1.5)) ** (1 / 2.2), rtol=1e-5)
