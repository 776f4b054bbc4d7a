"""The CPU oracle against the reference: golden vectors generated from the
reference's own shader code (tests/golden/make_golden.py) and, where the
reference tree is present, a live comparison with it."""
import os

import math

import numpy as np
import pytest

from asuna_gb300 import scenes
from oracle import oracle_py
from tests.golden.make_golden import CASES

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_rng_known_answers():
    g = np.load(os.path.join(GOLDEN, "rng_kat.npz"))
    L = oracle_py.port()
    import ctypes as C

    for (x, y, z), h in zip(g["xyz"], g["hash"]):
        assert L.oracle_xxhash32(int(x), int(y), int(z)) == int(h)
    for s, row in zip(g["seeds"], g["rand"]):
        st = C.c_uint32(int(s))
        got = np.array([L.oracle_rand(C.byref(st)) for _ in range(len(row))], np.float32)
        assert np.array_equal(got, row)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_golden(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    b, shot = CASES[name]()
    shot.depth_out_channel = -1
    film, rec, st = oracle_py.OracleScene(b.desc()).render(shot)
    # the reference's payload holds the clamped radiance (rgen:147)
    assert np.array_equal(np.clip(rec["radiance"], 0, 10), g["radiance"])
    for k in ("depth", "signature", "events", "shadows"):
        assert np.array_equal(rec[k], g[k]), k
    assert np.array_equal(film, g["film"])
    assert st["extend_rays"] > st["paths"] and st["shadow_rays"] > 0


@pytest.mark.skipif(oracle_py.ref() is None, reason="reference tree not present")
def test_oracle_matches_reference_live():
    b, shot = scenes.plugin_scene(40, 30, frames=4, max_depth=6, env=True, seed=23)
    shot.depth_out_channel = -1
    d = b.desc()
    film, rec, _ = oracle_py.OracleScene(d).render(shot)
    rfilm, rrec = oracle_py.ref_render(d, shot, threads=1)
    assert np.array_equal(np.clip(rec["radiance"], 0, 10), rrec["radiance"])
    assert np.array_equal(rec["signature"], rrec["signature"])
    assert np.array_equal(film, rfilm)


def test_oracle_resume_equals_single_call():
    b, shot = scenes.box_scene(16, 16, frames=6, max_depth=5)
    o = oracle_py.OracleScene(b.desc())
    full, _, _ = o.render(shot, records=False)
    shot.frames = 2
    part, _, _ = o.render(shot, records=False)
    shot.frame0, shot.frames = 2, 4
    part, _, _ = o.render(shot, film=part, records=False)
    assert np.array_equal(full, part)


def test_oracle_double_precision_close_to_float():
    b, shot = scenes.box_scene(16, 16, frames=64, max_depth=6)
    o = oracle_py.OracleScene(b.desc())
    f32, _, _ = o.render(shot, records=False)
    px = np.arange(256, dtype=np.uint32)
    f64, _ = o.pixels_f64(shot, px)
    a = f32[0, ..., :3].reshape(-1, 3)
    assert np.abs(a.mean() - f64.mean()) < 0.02 * f64.mean()


@pytest.mark.parametrize("which,fn,lo,hi,ulps", [(0, np.sin, -7, 7, 1), (1, np.cos, -7, 7, 1), (2, np.exp, -20, 1, 1),
                                                 (3, np.arccos, -1, 1, 3), (4, None, -3, 3, 3),
                                                 (5, np.log2, 1e-6, 40, 3), (6, np.exp2, -30, 30, 2),
                                                 (7, "pow", 0.0, 1.0, 80), (8, np.log, 1e-6, 40, 3),
                                                 (9, np.tan, -1.5, 1.5, 3)])
def test_shared_math_accuracy(which, fn, lo, hi, ulps):
    """include/asuna_math.h (used by the CUDA kernels and the oracle) against
    double precision, in ulps of the float result (pow: bases in (0, 1],
    exponents 1..40)."""
    L = oracle_py.port()
    rng = np.random.default_rng(which)
    x = rng.uniform(lo, hi, 20000).astype(np.float32)
    y = rng.uniform(-3, 3, 20000).astype(np.float32)
    if fn == "pow":
        x = np.maximum(x, np.float32(0.3))
        y = rng.uniform(1, 40, 20000).astype(np.float32)
    got = np.array([L.oracle_math(which, float(a), float(b)) for a, b in zip(x, y)], np.float32)
    if fn == "pow":
        ref = np.power(x.astype(np.float64), y.astype(np.float64))
    else:
        ref = np.arctan2(x.astype(np.float64), y.astype(np.float64)) if fn is None else fn(x.astype(np.float64))
    d = np.abs(got.view(np.int32).astype(np.int64) - ref.astype(np.float32).view(np.int32).astype(np.int64))
    assert d.max() <= ulps


@pytest.mark.parametrize("albedo", [(1.0, 1.0, 1.0), (0.5, 0.7, 0.9)])
def test_furnace_closed_form(albedo):
    """A convex Lambertian under a uniform background colour, no env map and
    no lights: sampleLights takes no light sample (rchit_layouts.glsl:127-134,
    case "no env & light"), while the miss shader still weights the BSDF
    sample by the power heuristic against the uniform-sphere pdf
    (raytrace.default.rmiss:41-50).  The expected radiance of a hit is then
    albedo x background x 2 int_0^1 c^3 / (c^2 + 1/16) dc = albedo x
    background x (1 - ln 17 / 16): the reference's estimator, not an
    energy-conserving one.  Pixels that see only the background get it
    exactly."""
    b, shot, inside, outside = scenes.furnace_scene(albedo, 24, 24, frames=64)
    film, _, _ = oracle_py.OracleScene(b.desc()).render(shot, records=False)
    img = film[0][..., :3].astype(np.float64)
    expect = np.array(albedo) * (1.0 - math.log(17.0) / 16.0)
    got = img[inside].mean(0)
    sigma = img[inside].std(0) / math.sqrt(inside.sum())
    assert np.all(np.abs(got - expect) <= 4 * sigma + 1e-4), (got, expect, sigma)
    assert np.all(img[outside] == 1.0)


def test_oracle_host_helpers_match_the_library():
    """The oracle's own restatements of the diffuse-Fresnel integral
    (material.cpp:6-37) and the perspective camera (camera.cpp:28-99), which
    the reference arm of the benchmark builds its workload with, agree with
    the library's: the integral bit for bit, the matrices to float rounding."""
    import asuna_gb300 as ag
    from asuna_gb300 import _abi as A
    from asuna_gb300 import scene as sc

    for ior in (1.1, 1.33, 1.5, 2.4):
        assert oracle_py.OracleHelpers.diffuse_fresnel(ior) == sc._LibraryHelpers.diffuse_fresnel(ior)
    for eye, at, fov, w, h in [((0, 0, 3.9), (0, 0, 0), 40.0, 256, 256), ((30, 5, -12), (1, 2, 3), 55.0, 1920, 1080),
                               ((-3, 8, 1), (0, 0, 0), 20.0, 512, 300)]:
        cams = []
        for prov in (sc._LibraryHelpers, oracle_py.OracleHelpers):
            with sc.host_helpers(prov):
                cams.append(ag.perspective_camera(eye, at, (0, 1, 0), fov, w, h, aperture=0.05, focal_distance=7.0))
        a, b = cams
        assert a.type == b.type == A.CAMERA_PERSPECTIVE
        for f in ("camera_to_world", "raster_to_camera", "env_transform"):
            x, y = np.array(getattr(a, f)), np.array(getattr(b, f))
            assert np.allclose(x, y, rtol=2e-6, atol=1e-7), (f, x, y)
        assert (a.aperture, a.focal_distance) == (b.aperture, b.focal_distance)


def test_sun_and_sky_defaults_match_the_library():
    """The builder's sun & sky defaults (set without the library) equal the
    library's asuna_sun_and_sky_default (Scene::reset, scene.cpp:112-129)."""
    import ctypes as C

    from asuna_gb300 import _abi as A
    from asuna_gb300 import scene as sc

    a, b = A.SunAndSky(), A.SunAndSky()
    A.lib().asuna_sun_and_sky_default(C.byref(a))
    sc._default_sky(b)
    assert bytes(a) == bytes(b)


@pytest.mark.skipif(oracle_py.ref() is None, reason="reference shader library not built")
@pytest.mark.parametrize("tm,auto,extra", [(0, 0, {}), (1, 0, {}), (2, 0, {}), (3, 0, {}), (4, 0, {}), (5, 0, {}),
                                           (6, 0, {}), (6, 1, {}), (6, 3, {}),
                                           (6, 0, {"contrast": 1.3, "brightness": 0.8, "saturation": 0.6,
                                                   "vignette": 0.4, "avg_lum": 1.7}),
                                           (3, 0, {"zoom": 0.75})])
def test_oracle_tonemap_matches_reference_post_shader(tm, auto, extra):
    """The oracle's tone mapping (oracle_tonemap, the checker of the GPU's
    asuna_tonemap) equals the reference's own post.idle.frag compiled as
    host C++ (oracle/post_harness.cpp) bit for bit, for every operator, with
    and without auto / local exposure, with the custom operator's contrast,
    brightness, saturation and vignette, and with zoom; the sampler's mip
    chain and filtering are the harness's (the graphics driver's in the
    reference)."""
    import ctypes as C

    import asuna_gb300 as ag

    rng = np.random.default_rng(40 + tm + 10 * auto)
    img = np.exp(rng.normal(-0.5, 1.5, (48, 64, 4))).astype(np.float32)
    img[..., 3] = 1.0
    post = ag.default_post(tm)
    post.auto_exposure = auto
    for k, v in extra.items():
        setattr(post, k, v)
    a = np.zeros_like(img)
    b = np.zeros_like(img)
    assert oracle_py.port().oracle_tonemap(img.ctypes.data, 64, 48, C.byref(post), a.ctypes.data) == 0
    L = oracle_py.ref()
    L.ref_post.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    assert L.ref_post(img.ctypes.data, 64, 48, C.byref(post), b.ctypes.data) == 0
    assert np.array_equal(a, b), (np.abs(a - b).max(), (a != b).mean())
