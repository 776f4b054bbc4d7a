"""Generates the golden vectors of tests/golden/ from the reference's own
shader code compiled as host C++ (oracle/gen_ref.py + oracle/ref_harness.cpp).

Needs the reference tree (it is read where it lies; nothing of it is copied).
Writes small .npz fixtures: RNG known answers and per-path records + film
images of seeded procedural scenes.  Run: python tests/golden/make_golden.py
[case ...] (no argument: every fixture).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from asuna_gb300 import scenes  # noqa: E402
from oracle import oracle_py  # noqa: E402

CASES = {
    "box_32x32x4": lambda: scenes.box_scene(32, 32, frames=4, max_depth=8, channels=("albedo", "normal")),
    "plugins_env_48x32x3": lambda: scenes.plugin_scene(48, 32, frames=3, env=True,
                                                       channels=("albedo", "normal", "position", "uv", "tangent",
                                                                 "roughness", "specular")),
    "plugins_bg_opencv_32x24x2": lambda: scenes.plugin_scene(32, 24, frames=2, env=False, opencv=True,
                                                             channels=("albedo", "normal")),
    "plugins_textured_40x28x2": lambda: scenes.plugin_scene(40, 28, frames=2, env=True, textured=True,
                                                            channels=("albedo", "normal", "tangent", "roughness",
                                                                      "specular", "uv")),
    "plugins_opacity_40x28x3": lambda: scenes.plugin_scene(40, 28, frames=3, env=True, textured=True, opacity=True,
                                                           channels=("albedo", "normal", "depth")),
    "sky_day_48x32x3": lambda: scenes.sky_scene(48, 32, frames=3, channels=("albedo", "normal")),
    "sky_dusk_light_40x24x2": lambda: scenes.sky_scene(40, 24, frames=2, dusk=True, point_light=True,
                                                       channels=("albedo", "normal")),
}


def rng_kat():
    L = oracle_py.ref()
    rs = np.random.default_rng(5)
    xyz = rs.integers(0, 2**32, size=(256, 3), dtype=np.uint64).astype(np.uint32)
    xyz[:16] = [[x, y, z] for x, y, z in zip(range(16), range(0, 32, 2), [0] * 8 + [1] * 8)]
    h = np.array([L.ref_xxhash32(int(a), int(b), int(c)) for a, b, c in xyz], np.uint32)
    seeds = h[:16].copy()
    draws = np.zeros((16, 64), np.float32)
    for i, s in enumerate(seeds):
        st = C.c_uint32(int(s))
        for k in range(64):
            draws[i, k] = L.ref_rand(C.byref(st))
    return dict(xyz=xyz, hash=h, seeds=seeds, rand=draws)


def main(argv=None):
    """Regenerates every fixture, or only the cases named on the command line."""
    names = list(argv if argv is not None else sys.argv[1:]) or list(CASES)
    if oracle_py.ref() is None:
        print("reference tree not found; golden vectors not regenerated", file=sys.stderr)
        return 2
    if not argv and len(sys.argv) <= 1:
        np.savez_compressed(os.path.join(HERE, "rng_kat.npz"), **rng_kat())
    for name in names:
        make = CASES[name]
        b, shot = make()
        shot.depth_out_channel = -1  # the reference has no depth channel
        film, rec = oracle_py.ref_render(b.desc(), shot, threads=1)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), film=film, radiance=rec["radiance"],
                            depth=rec["depth"], signature=rec["signature"], events=rec["events"],
                            shadows=rec["shadows"])
        print(name, rec.shape, float(film[0, ..., :3].mean()))
    return 0


if __name__ == "__main__":
    sys.exit(main())
