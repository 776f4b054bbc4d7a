"""Parity statistics of GPU path records against the CPU oracle (test
infrastructure: used by the tests and by the benchmark's parity check).

Tolerance: a path agrees when every radiance channel satisfies
|gpu - oracle| <= 1e-4 * |oracle| + 1e-6 (relative 1e-4 with an absolute floor
for near-black paths).  A branch flip is a path whose hit/lobe signature,
shadow-ray set or visibility bits differ (the two took different branches).
"""
import numpy as np

REL = 1e-4
ABS = 1e-6


def compare(rec, orec):
    a, r = rec["radiance"], orec["radiance"]
    within = np.all(np.abs(a - r) <= REL * np.abs(r) + ABS, axis=1)
    flips = (rec["signature"] != orec["signature"]) | (rec["events"] != orec["events"]) | \
            (rec["shadows"] != orec["shadows"]) | (rec["depth"] != orec["depth"])
    return {"paths": int(len(rec)), "within": float(within.mean()), "exact": float(np.all(a == r, axis=1).mean()),
            "flips": int(flips.sum()), "flip_frac": float(flips.mean()),
            "outside_without_flip": int((~within & ~flips).sum())}


def sample_parity(ctx, scene, desc, shot, npixels=16384, frames=4, seed=0, oracle_scene=None):
    """GPU path records against the oracle's on a seeded subset of a shot's
    pixels over frames [0, frames): the GPU renders the whole shot through
    asuna_render_paths, the oracle only the subset; returns compare() of the
    subset's records plus the sample's size."""
    import copy

    from oracle import oracle_py

    rng = np.random.default_rng(seed)
    npix = shot.width * shot.height
    px = np.sort(rng.choice(npix, size=min(npixels, npix), replace=False)).astype(np.uint32)
    s = copy.copy(shot)
    s.frames, s.frame0 = frames, 0
    film = ctx.create_film(s.width, s.height)
    rec = ctx.render_paths(scene, s, film).reshape(frames, npix)[:, px].reshape(-1)
    film.close()
    osc = oracle_scene if oracle_scene is not None else oracle_py.OracleScene(desc)
    _, orec, _ = osc.render(s, records=True, pixels=px)
    if oracle_scene is None:
        osc.close()
    out = compare(rec, orec)
    out.update({"pixels": int(len(px)), "frames": frames})
    return out
