"""GPU path records and films against the CPU oracle (same seeded inputs).

Tolerance (stated in tests/parity.py): per path every radiance channel within
1e-4 relative (+1e-6 absolute); at least 99.9% of paths must agree; paths
that took a different branch (hit / lobe / visibility signature) are counted
as flips and reported.  Integer parts (RNG streams, depths, signatures) are
compared bit for bit on the paths without flips.
"""
import numpy as np
import pytest

from asuna_gb300 import scenes
from oracle import oracle_py
from tests.parity import compare

pytestmark = pytest.mark.gpu


def _run(ctx, b, shot):
    d = b.desc()
    scene = ctx.create_scene(d)
    film = ctx.create_film(shot.width, shot.height)
    rec = ctx.render_paths(scene, shot, film)
    imgs = np.stack([film.read(k) for k in range(9)])
    ofilm, orec, _ = oracle_py.OracleScene(d).render(shot)
    return rec, orec, imgs, ofilm


def _check(rec, orec, imgs, ofilm, film_tol=1e-3):
    c = compare(rec, orec)
    print(c)
    assert c["within"] >= 0.999, c
    same = (rec["signature"] == orec["signature"]) & (rec["events"] == orec["events"])
    assert np.array_equal(rec["depth"][same], orec["depth"][same])
    # films: radiance, AOVs and weight sums
    assert np.abs(imgs[8] - ofilm[8]).max() <= 1e-5
    err = np.abs(imgs[0] - ofilm[0])
    assert np.quantile(err, 0.999) <= film_tol
    return c


def test_box_scene_small(ctx):
    b, shot = scenes.box_scene(64, 64, frames=4, max_depth=8)
    rec, orec, imgs, ofilm = _run(ctx, b, shot)
    c = _check(rec, orec, imgs, ofilm)
    assert c["exact"] > 0.5  # FP32 arithmetic in the same order: most paths are bit-identical
    for k in (1, 2, 3):  # albedo, normal, depth AOVs
        assert np.quantile(np.abs(imgs[k] - ofilm[k]), 0.999) <= 1e-4


def test_box_scene_full_config(ctx):
    # the small-box configuration: 256x256, 16 spp (frames), depth 8
    b, shot = scenes.box_scene(256, 256, frames=16, max_depth=8)
    rec, orec, imgs, ofilm = _run(ctx, b, shot)
    _check(rec, orec, imgs, ofilm)


@pytest.mark.parametrize("env,opencv", [(True, False), (False, True), (True, True)])
def test_every_plugin(ctx, env, opencv):
    b, shot = scenes.plugin_scene(96, 64, frames=4, max_depth=8, env=env, opencv=opencv)
    rec, orec, imgs, ofilm = _run(ctx, b, shot)
    _check(rec, orec, imgs, ofilm, film_tol=5e-3)


@pytest.mark.parametrize("face_normal,opacity", [(0, False), (1, False), (0, True)])
def test_every_plugin_textured(ctx, face_normal, opacity):
    """Every texture slot the shaders read (diffuse, alpha, metalness and
    roughness, specular, tangent- and object-space normal maps, tangent map,
    emissive radiance); with use_face_normal the normal maps must have no
    effect, as configureShadingFrame puts the geometric normal back.  With
    `opacity`, PBR / Disney (mask texture) / kang18 pass rays through
    without counting a bounce, which the wavefront tracks per path."""
    b, shot = scenes.plugin_scene(96, 64, frames=4, max_depth=8, env=True, textured=True, opacity=opacity,
                                  channels=("albedo", "normal", "tangent", "roughness", "specular", "uv"))
    shot.state.use_face_normal = face_normal
    rec, orec, imgs, ofilm = _run(ctx, b, shot)
    _check(rec, orec, imgs, ofilm, film_tol=5e-3)


def test_mixed_scene_small(ctx):
    b, shot = scenes.mixed_scene(160, 90, frames=2, max_depth=12, n_spheres=12, level=4, seed=3, rr_depth=3,
                                 env_size=(128, 64))
    rec, orec, imgs, ofilm = _run(ctx, b, shot)
    _check(rec, orec, imgs, ofilm, film_tol=5e-2)


@pytest.mark.parametrize("albedo", [(1.0, 1.0, 1.0), (0.5, 0.7, 0.9)])
def test_furnace_closed_form(ctx, albedo):
    """The GPU on the furnace of tests/test_oracle.py: hits converge to
    albedo x (1 - ln 17 / 16) (the reference's estimator without a light
    sample), background pixels are exactly the background, and the film
    equals the oracle's within the parity tolerance."""
    import math

    b, shot, inside, outside = scenes.furnace_scene(albedo, 48, 48, frames=256)
    rec, orec, imgs, ofilm = _run(ctx, b, shot)
    _check(rec, orec, imgs, ofilm)
    img = imgs[0][..., :3].astype(np.float64)
    expect = np.array(albedo) * (1.0 - math.log(17.0) / 16.0)
    got = img[inside].mean(0)
    sigma = img[inside].std(0) / math.sqrt(inside.sum())
    assert np.all(np.abs(got - expect) <= 4 * sigma + 1e-4), (got, expect, sigma)
    assert np.all(img[outside] == 1.0)


@pytest.mark.parametrize("dusk,light", [(False, False), (True, True)], ids=["day", "dusk_light"])
def test_sun_and_sky(ctx, dusk, light):
    """The sun & sky environment (GpuSunAndSky in use) in the miss shading
    and the environment light sample: by day with the sun disk in view, and
    at dusk (sun below the horizon, haze, shifted colours, raised and blurred
    horizon) with a point light sharing the light sample."""
    b, shot = scenes.sky_scene(64, 48, frames=4, dusk=dusk, point_light=light)
    rec, orec, imgs, ofilm = _run(ctx, b, shot)
    c = _check(rec, orec, imgs, ofilm)
    assert c["exact"] > 0.5


@pytest.fixture(scope="module")
def benchmark_workload(ctx):
    """The benchmarked configuration itself: 64 level-7 icospheres
    (20,971,520 triangles + ground + 4 light triangles), 1920x1080, depth 12,
    1024x512 lognormal environment with a x1000 hotspot, 4 triangle lights,
    aperture 0.05; the scene seed of bench.py."""
    b, shot = scenes.mixed_scene(1920, 1080, frames=4, max_depth=12, n_spheres=64, level=7, seed=1234, rr_depth=3)
    d = b.desc()
    scene = ctx.create_scene(d)
    osc = oracle_py.OracleScene(d)
    yield b, d, shot, scene, osc
    osc.close()
    scene.close()


@pytest.mark.parametrize("rr", [True, False], ids=["rr3", "rr_off"])
def test_benchmark_workload_parity(ctx, benchmark_workload, rr):
    """Per-path parity on the 21M-triangle 1080p benchmark workload: a seeded
    subset of 16,384 pixels x 4 frames (65,536 paths), once with Russian
    roulette after depth 3 as benchmarked and once without it (the
    reference's estimator); every radiance channel within 1e-4 relative on
    >= 99.9% of paths, branch flips counted and bounded."""
    import copy

    from asuna_gb300 import _abi as A
    from oracle import parity

    b, d, shot, scene, osc = benchmark_workload
    s = copy.copy(shot)
    if not rr:
        s.flags &= ~A.SHOT_RR
    c = parity.sample_parity(ctx, scene, d, s, npixels=16384, frames=4, seed=0, oracle_scene=osc)
    print(c)
    assert c["paths"] == 65536
    assert c["within"] >= 0.999, c
    assert c["flip_frac"] <= 1e-3, c
