"""The serving driver's host logic (asuna_gb300.serving.poisson_load) on a
fake server (no GPU): Poisson submission order, every result collected,
kept films read before their release, every film released once, and the
latency / throughput summary computed from the server's own timestamps."""
import types

import numpy as np

from asuna_gb300 import _abi as A
from asuna_gb300.serving import poisson_load


class FakeServer:
    """Finishes request k `lat[k]` seconds after its arrival (server clock =
    submission order); every fifth request is rejected."""

    def __init__(self, lat):
        self.lat = lat
        self.submitted, self.released, self.read_ids, self.flags = [], [], [], []
        self.clock = 0.0
        self.pending = []

    def submit(self, scene, shot, denoise=False):
        rid = 100 + len(self.submitted)
        k = len(self.submitted)
        self.submitted.append(rid)
        self.flags.append(denoise)
        arrival = 0.01 * k
        ok = k % 5 != 4
        self.pending.append({"id": rid, "status": A.OK if ok else A.ERR_BUSY, "arrival_s": arrival,
                             "start_s": arrival + (0.02 if k % 2 else 0.0), "finish_s": arrival + self.lat[k],
                             "samples": shot.width * shot.height * shot.spp if ok else 0})
        return rid

    def poll(self):
        out, self.pending = self.pending, []
        return out

    def read(self, rid, w, h, image=0):
        assert rid not in self.released
        self.read_ids.append(rid)
        return np.full((h, w, 4), float(rid), np.float32)

    def release(self, rid):
        assert rid not in self.released
        self.released.append(rid)


def test_poisson_load_on_a_fake_server():
    n = 40
    lat = np.linspace(0.05, 0.45, n)
    srv = FakeServer(lat)
    shots = [types.SimpleNamespace(width=4, height=2, spp=16) for _ in range(n)]
    reqs = [(0, s) for s in shots]
    out = poisson_load(srv, reqs, rate_hz=4000.0, seed=1, keep=[0, 3, 4], denoise=[k % 3 == 0 for k in range(n)])
    ok = [k for k in range(n) if k % 5 != 4]
    assert out["requests"] == n and out["completed"] == len(ok) and out["rejected"] == n - len(ok)
    assert out["missing"] == 0 and abs(out["rejection_rate"] - (n - len(ok)) / n) < 1e-12
    assert sorted(srv.released) == srv.submitted  # every film released exactly once
    assert srv.flags == [k % 3 == 0 for k in range(n)]
    # kept films are read before their release; a rejected one (index 4) has none
    assert set(out["films"]) == {0, 3} and srv.read_ids == [100, 103]
    assert float(out["films"][3][0, 0, 0]) == 103.0
    lats = lat[ok]
    assert abs(out["p50_s"] - np.percentile(lats, 50)) < 1e-9
    assert abs(out["p99_s"] - np.percentile(lats, 99)) < 1e-9
    span = max(0.01 * k + lat[k] for k in ok) - min(0.01 * k for k in ok)
    assert abs(out["msamples_per_s"] - len(ok) * 4 * 2 * 16 / span / 1e6) < 1e-9
    assert abs(out["queued_frac"] - np.mean([k % 2 == 1 for k in ok])) < 1e-12
