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
                                                 (7, "pow", 0.0, 1.0, 80), (8, np.log, 1e-6, 40, 3)])
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
