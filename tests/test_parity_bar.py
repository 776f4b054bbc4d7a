"""The parity bar itself (host only, no GPU): oracle.parity.compare counts a
path as agreeing only within its stated tolerance and reports a changed
branch as a flip.  The mistakes are planted in a copy of the oracle's own
records, so the bar is checked on the CPU against known answers."""
import numpy as np

from asuna_gb300 import scenes
from oracle import oracle_py, parity


def _records():
    b, shot = scenes.box_scene(16, 16, frames=2, max_depth=5)
    o = oracle_py.OracleScene(b.desc())
    try:
        _, rec, _ = o.render(shot, records=True)
    finally:
        o.close()
    return rec.reshape(-1)


def test_identical_records_agree_exactly():
    rec = _records()
    out = parity.compare(rec, rec.copy())
    assert out == {"paths": len(rec), "within": 1.0, "exact": 1.0, "flips": 0, "flip_frac": 0.0,
                   "outside_without_flip": 0}


def test_planted_mistakes_are_caught():
    rec = _records()
    bright = np.nonzero(np.max(rec["radiance"], axis=1) > 0.1)[0]
    assert len(bright) >= 3
    a, b_, c = bright[:3]
    got = rec.copy()
    # inside the bar: a relative change well below 1e-4
    got["radiance"][a] *= 1.0 + 2e-5
    # outside it: a relative change of 1e-3 on one channel, same branches
    got["radiance"][b_, 0] *= 1.001
    # a changed branch: another hit/lobe signature
    got["signature"][c] ^= 1
    out = parity.compare(got, rec)
    n = len(rec)
    assert out["flips"] == 1 and out["outside_without_flip"] == 1
    assert abs(out["within"] - (n - 1) / n) < 1e-12
    assert abs(out["exact"] - (n - 2) / n) < 1e-12
    # a path darker than the absolute floor agrees however it changes relatively
    dark = np.nonzero(np.max(np.abs(rec["radiance"]), axis=1) == 0)[0]
    if len(dark):
        got2 = rec.copy()
        got2["radiance"][dark[0]] = 5e-7
        assert parity.compare(got2, rec)["within"] == 1.0
