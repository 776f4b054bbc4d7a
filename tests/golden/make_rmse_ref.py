"""FP64 reference of the 1080p benchmark workload on a seeded pixel subset.

Renders the mixed-material scene (64 level-7 spheres, 1920x1080, depth 12,
Russian roulette past depth 3) with the double-precision CPU oracle at
262,144 samples per pixel for 1,024 seeded pixels, with a sample stream
(seed 12345) independent of the GPU renders it judges.  Stores the per-pixel
mean radiance and the variance of that mean; an RMSE against this reference
subtracts the reference's own variance.  Used by bench.py --denoise-rmse.

Usage: python tests/golden/make_rmse_ref.py [--spp N] [--pixels N]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from asuna_gb300 import scenes  # noqa: E402
from oracle import oracle_py  # noqa: E402


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--spp", type=int, default=262144)
    ap.add_argument("--pixels", type=int, default=1024)
    ap.add_argument("--out", default=os.path.join(HERE, "rmse_ref_mixed_1080p.npz"))
    a = ap.parse_args(argv)
    b, shot = scenes.mixed_scene()
    o = oracle_py.OracleScene(b.desc())
    px = np.sort(np.random.default_rng(99).choice(shot.width * shot.height, a.pixels, replace=False))
    px = px.astype(np.uint32)
    shot.frame0 = 0
    shot.frames = a.spp
    shot.seed = 12345
    t = time.time()
    mean, var, st = o.pixels_f64(shot, px, variance=True)
    np.savez_compressed(a.out, pixels=px, mean=mean, var=var, spp=a.spp, seed=12345, width=shot.width,
                        height=shot.height, seconds=time.time() - t, threads=st["threads"])
    print(f"{a.out}: {a.pixels} px x {a.spp} spp in {time.time() - t:.0f} s; mean {mean.mean():.4f}, "
          f"reference RMS noise {np.sqrt(var.mean()):.5f}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
