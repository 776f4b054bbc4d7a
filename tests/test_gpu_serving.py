"""Continuous-batching render server: a request renders the same film alone
and mixed with concurrent requests of other scenes, resolutions and spp;
admission rejects what cannot be served and reports why; nothing faults."""
import numpy as np
import pytest

import asuna_gb300 as ag
from asuna_gb300 import _abi as A
from asuna_gb300 import scenes
from asuna_gb300.serving import Server, poisson_load

pytestmark = pytest.mark.gpu


def _shot(make, w, h, frames, seed=0):
    _, s = make(w, h, frames)
    s.seed = seed
    return s


def test_result_same_alone_and_in_the_mix():
    b1, base1 = scenes.plugin_scene(64, 48, frames=6, max_depth=6)
    b2, base2 = scenes.box_scene(48, 40, frames=3, max_depth=6)
    srv = Server(slots=2, frames_per_chunk=2, max_batch=4)
    try:
        s1, s2 = srv.add_scene(b1.desc()), srv.add_scene(b2.desc())
        alone = poisson_load(srv, [(s1, base1)], rate_hz=1000.0, keep=[0])["films"][0]
        mix = []
        for k in range(10):
            if k % 3 == 0:
                _, sh = scenes.box_scene(32 + 8 * k, 24 + 4 * k, frames=1 + k % 4, max_depth=6)
                mix.append((s2, sh))
            else:
                _, sh = scenes.plugin_scene(40 + 4 * k, 32, frames=2 + k % 5, max_depth=6)
                sh.seed = k
                mix.append((s1, sh))
        mix.insert(4, (s1, base1))
        out = poisson_load(srv, mix, rate_hz=200.0, keep=[4])
        assert out["completed"] == len(mix) and out["rejected"] == 0
        assert np.array_equal(out["films"][4], alone)
    finally:
        srv.close()
    # and the same as a plain render call
    ctx = ag.Context(0)
    sc = ctx.create_scene(b1.desc())
    f = ctx.create_film(64, 48)
    ctx.render(sc, base1, f)
    assert np.array_equal(f.read(0), alone)


def test_admission_rejections_are_reported():
    b, shot = scenes.box_scene(32, 32, frames=2, max_depth=4)
    srv = Server(slots=1, frames_per_chunk=1, max_queue=2, memory_budget=64 << 20)
    try:
        sid = srv.add_scene(b.desc())
        bad = srv.submit(sid + 5, shot)  # unknown scene
        _, big = scenes.box_scene(4096, 4096, frames=1, max_depth=4)  # film larger than the budget
        huge = srv.submit(sid, big)
        for _ in range(12):
            srv.submit(sid, shot)
        srv.drain(120.0)
        res = {}
        for _ in range(50):
            for r in srv.poll():
                res[r["id"]] = r
            if len(res) >= 14:
                break
        assert res[bad]["status"] == A.ERR_INVALID
        assert res[huge]["status"] == A.ERR_OOM
        busy = sum(1 for r in res.values() if r["status"] == A.ERR_BUSY)
        done = sum(1 for r in res.values() if r["status"] == A.OK)
        assert busy >= 1 and done >= 2 and busy + done == 12
        st = srv.stats()
        assert st["rejected"] == 2 + busy and st["pending"] == 0
    finally:
        srv.close()
