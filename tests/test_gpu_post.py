"""Post pass and offline outputs on the GPU: asuna_tonemap against the
oracle's restatement of post.idle.frag for every operator (8-bit output
within one step), and asuna_tracer_run_offline's files (tone-mapped
_shot_%04d.png, or _shot_%04d.exr with output_hdr, plus AOV channels)
against the film they come from."""
import json
import struct
import zlib

import numpy as np
import pytest

import asuna_gb300 as ag
from asuna_gb300 import _abi as A
from asuna_gb300 import scenes
from oracle import oracle_py
import ctypes as C

pytestmark = pytest.mark.gpu


def to8(x):
    return np.clip(np.asarray(x, np.float32), 0.0, 1.0) * np.float32(255.0) + np.float32(0.5)


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    assert not raw[:, 0].any()  # filter type 0 on every row
    return raw[:, 1:].reshape(h, w, 4)


def read_exr(path, w, h):
    """Uncompressed scanline FLOAT RGBA: the offset table follows the header's
    terminating null byte; each chunk = y, size, then A, B, G, R rows."""
    data = open(path, "rb").read()
    assert data[:4] == b"\x76\x2f\x31\x01"
    pos = 8
    while data[pos] != 0:  # attributes: name\0 type\0 size data
        pos = data.index(b"\0", pos) + 1
        pos = data.index(b"\0", pos) + 1
        n, = struct.unpack("<i", data[pos:pos + 4])
        pos += 4 + n
    pos += 1 + 8 * h
    img = np.zeros((h, w, 4), np.float32)
    for _ in range(h):
        y, size = struct.unpack("<ii", data[pos:pos + 8])
        rows = np.frombuffer(data[pos + 8:pos + 8 + size], np.float32).reshape(4, w)
        img[y] = rows[[3, 2, 1, 0]].T
        pos += 8 + size
    return img


@pytest.fixture(scope="module")
def film_and_ctx():
    ctx = ag.Context(0)
    b, shot = scenes.plugin_scene(64, 48, frames=4, max_depth=6)
    scene = ctx.create_scene(b.desc())
    f = ctx.create_film(64, 48)
    ctx.render(scene, shot, f)
    return ctx, f


CASES = [(t, 0, {}) for t in range(6)] + [
    (A.TONEMAP_CUSTOM, 0, {}),
    (A.TONEMAP_CUSTOM, 1, {"contrast": 1.2, "saturation": 0.8, "vignette": 0.3, "brightness": 1.1}),
    (A.TONEMAP_CUSTOM, 3, {"key": 0.3, "avg_lum": 1.5}),
]


@pytest.mark.parametrize("tm,auto,extra", CASES)
def test_tonemap_matches_oracle(film_and_ctx, tm, auto, extra):
    ctx, film = film_and_ctx
    post = ag.default_post(tm)
    post.auto_exposure = auto
    for k, v in extra.items():
        setattr(post, k, v)
    got = ctx.tonemap(film, 0, post)
    hdr = film.read(0)
    ref = np.zeros_like(hdr)
    L = oracle_py.port()
    assert L.oracle_tonemap(hdr.ctypes.data, 64, 48, C.byref(post), ref.ctypes.data) == 0
    # auto exposure divides by the pixel's luminance (post.idle.frag:45,68):
    # a black pixel gives 0/0 there, which the contrast clamp (minNum /
    # maxNum, as the hardware evaluates GLSL clamp) turns into 0
    assert np.isfinite(got[..., :3]).all() and np.isfinite(ref[..., :3]).all()
    black = np.all(hdr[..., :3] == 0, axis=-1)
    if auto and black.any():
        assert np.all(got[black][:, :3] == 0) and np.all(ref[black][:, :3] == 0)
    a, b = to8(got[..., :3]).astype(np.int32), to8(ref[..., :3]).astype(np.int32)
    assert np.abs(a - b).max() <= 1
    assert np.mean(a == b) >= 0.999
    assert np.array_equal(got[..., 3], hdr[..., 3])


def _box_scene_file(tmp_path, output_hdr):
    obj = tmp_path / "quad.obj"
    obj.write_text("v -1 -1 0\nv 1 -1 0\nv 1 1 0\nv -1 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\nf 1//1 3//1 4//1\n")
    scene = {
        "state": {"path_tracing": {"spp": 3, "max_path_depth": 4, "multi_channel": ["albedo", "normal"],
                                   "multi_channel_ldr": [True, False]},
                  "post_processing": {"tone_mapping": "Aces"}, "output_hdr": output_hdr},
        "camera": {"type": "perspective", "fov": 45.0, "film": {"resolution": [40, 32]}},
        "materials": [{"type": "brdf_lambertian", "name": "white", "diffuse_reflectance": [0.7, 0.6, 0.5]}],
        "lights": [{"type": "point", "position": [0, 0, 2], "radiance": [4, 4, 4]}],
        "meshes": [{"name": "quad", "path": "quad.obj"}],
        "instances": [{"mesh": "quad", "material": "white"}],
        "shots": [{"type": "lookat", "eye": [0, 0, 3], "lookat": [0, 0, 0], "up": [0, 1, 0]}],
    }
    path = tmp_path / "scene.json"
    path.write_text(json.dumps(scene))
    return str(path)


@pytest.mark.parametrize("output_hdr", [False, True])
def test_offline_outputs(tmp_path, output_hdr):
    path = _box_scene_file(tmp_path, output_hdr)
    ctx = ag.Context(0)
    prefix = str(tmp_path / "out")
    ctx.run_offline(path, prefix)
    js = ag.JsonScene(path)
    scene = ctx.create_scene(js.desc())
    shot = js.shots()[0]
    f = ctx.create_film(40, 32)
    ctx.render(scene, shot, f)
    post = A.PostState()
    A.check(A.lib().asuna_json_post_state(js.handle, C.byref(post)))
    assert post.tm_type == A.TONEMAP_ACES
    if output_hdr:
        assert np.array_equal(read_exr(prefix + "_shot_0000.exr", 40, 32), f.read(0))
    else:
        png = read_png(prefix + "_shot_0000.png")
        want = to8(ctx.tonemap(f, 0, post)).astype(np.uint8)
        assert np.array_equal(png, want)
    # AOV channels: albedo as PNG (multi_channel_ldr), normal as EXR
    assert np.array_equal(read_png(prefix + "_shot_0000_channel_0000.png"), to8(f.read(1)).astype(np.uint8))
    assert np.array_equal(read_exr(prefix + "_shot_0000_channel_0001.exr", 40, 32), f.read(2))


def test_offline_scanline_outputs(tmp_path):
    """--output_scanline (tracer.cpp:347-395): the AOV channels as [n, 3]
    float32 .npy arrays (under their image names) of the pixels whose first
    channel has .z == 1, the first channel's .z holding the pixel index."""
    obj = tmp_path / "quad.obj"
    obj.write_text("v -1 -1 0\nv 1 -1 0\nv 1 1 0\nv -1 1 0\nvn 0 0 1\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
                   "f 1/1/1 2/2/1 3/3/1\nf 1/1/1 3/3/1 4/4/1\n")
    scene = {
        "state": {"path_tracing": {"spp": 2, "max_path_depth": 3, "multi_channel": ["uv", "normal"]},
                  "output_hdr": True},
        "camera": {"type": "perspective", "fov": 45.0, "film": {"resolution": [40, 32]}},
        "materials": [{"type": "brdf_lambertian", "name": "white", "diffuse_reflectance": [0.7, 0.6, 0.5]}],
        "lights": [{"type": "point", "position": [0, 0, 2], "radiance": [4, 4, 4]}],
        "meshes": [{"name": "quad", "path": "quad.obj"}],
        "instances": [{"mesh": "quad", "material": "white"}],
        "shots": [{"type": "lookat", "eye": [0, 0, 4], "lookat": [0, 0, 0], "up": [0, 1, 0]}],
    }
    path = tmp_path / "scene.json"
    path.write_text(json.dumps(scene))
    ctx = ag.Context(0)
    prefix = str(tmp_path / "out")
    ctx.run_offline(str(path), prefix, output_scanline=True)
    js = ag.JsonScene(str(path))
    f = ctx.create_film(40, 32)
    ctx.render(ctx.create_scene(js.desc()), js.shots()[0], f)
    uv, nrm = f.read(1).reshape(-1, 4), f.read(2).reshape(-1, 4)
    valid = np.nonzero(uv[:, 2] == 1.0)[0]
    assert 0 < valid.size < 40 * 32  # the quad covers part of the frame
    a = np.load(prefix + "_shot_0000_channel_0000.exr")
    b = np.load(prefix + "_shot_0000_channel_0001.exr")
    assert a.dtype == np.float32 and a.shape == (valid.size, 3) and b.shape == (valid.size, 3)
    assert np.array_equal(a[:, :2], uv[valid, :2]) and np.array_equal(a[:, 2], valid.astype(np.float32))
    assert np.array_equal(b, nrm[valid, :3])
    # the shot image itself stays an image
    assert np.array_equal(read_exr(prefix + "_shot_0000.exr", 40, 32), f.read(0))
