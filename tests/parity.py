"""Parity statistics of GPU path records against the CPU oracle.

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
