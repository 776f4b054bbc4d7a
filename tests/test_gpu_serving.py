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


def test_registered_scenes_built_on_admission_and_evicted():
    """Scenes registered with the server are built when their first request
    is admitted and charged to the memory budget; with room for only one of
    them, requests alternating between two scenes make the server drop the
    idle one (least recently used) and rebuild it later.  Results equal
    plain renders."""
    b1, _ = scenes.mixed_scene(64, 64, frames=1, n_spheres=8, level=4, seed=21, env_size=(64, 32))
    b2, _ = scenes.mixed_scene(64, 64, frames=1, n_spheres=8, level=4, seed=22, env_size=(64, 32))
    d1, d2 = b1.desc(), b2.desc()
    ctx = ag.Context(0)
    size = max(ctx.create_scene(d).stats()["device_bytes"] for d in (d1, d2))
    shots = [scenes.mixed_shot(b, 48, 32, 3, seed=k) for k, b in enumerate((b1, b2, b1, b2))]
    # room for one scene (and its estimate) and a few films, not two scenes
    srv = Server(slots=1, frames_per_chunk=2, max_batch=2, memory_budget=int(1.6 * size) + (4 << 20))
    try:
        s1, s2 = srv.register_scene(d1), srv.register_scene(d2)
        reqs = [(s1 if k % 2 == 0 else s2, sh) for k, sh in enumerate(shots)]
        out = poisson_load(srv, reqs, rate_hz=5.0, keep=[0, 1, 2, 3])
        st = srv.stats()
        assert out["completed"] == 4 and out["rejected"] == 0
        assert st["scenes_built"] >= 3 and st["scenes_evicted"] >= 2
        assert st["scene_bytes"] <= int(1.6 * size) + (4 << 20)
    finally:
        srv.close()
    for k, (b, sh) in enumerate(zip((b1, b2, b1, b2), shots)):
        sc = ctx.create_scene(b.desc())
        f = ctx.create_film(48, 32)
        ctx.render(sc, sh, f)
        assert np.array_equal(f.read(0), out["films"][k])


def test_denoised_request_same_alone_and_in_the_mix():
    """A request with the denoise flag renders its frames as two halves and
    returns asuna_denoise_blended of them; alone, in a mix with plain and
    denoised requests of other resolutions, and through the library's own
    calls, the result is the same (1e-6 relative: the blend weight comes
    from double-precision sums whose order varies)."""
    from asuna_gb300 import denoise as dn

    b, shot = scenes.plugin_scene(64, 48, frames=6, max_depth=6, channels=("albedo", "normal"))
    ctx = ag.Context(0)
    net = dn.Denoiser(ctx, seed=3, max_pixels=64 * 64)
    params = net.get_params()
    srv = Server(slots=2, frames_per_chunk=2, max_batch=3)
    try:
        srv.set_denoiser(params, max_pixels=128 * 128)
        sid = srv.add_scene(b.desc())
        reqs = [(sid, shot, True)]
        alone_id = srv.submit(sid, shot, denoise=True)
        srv.drain(120.0)
        res = {r["id"]: r for r in srv.poll()}
        assert res[alone_id]["status"] == A.OK
        alone = srv.read(alone_id, 64, 48, 0)
        srv.release(alone_id)
        ids = []
        for k in range(8):
            _, sh = scenes.plugin_scene(40 + 8 * k, 32, frames=2 + k % 4, max_depth=6, channels=("albedo", "normal"))
            sh.seed = 10 + k
            ids.append(srv.submit(sid, sh, denoise=(k % 2 == 0)))
            if k == 3:
                mixed_id = srv.submit(sid, shot, denoise=True)
        srv.drain(120.0)
        res = {r["id"]: r for r in srv.poll()}
        assert all(res[i]["status"] == A.OK for i in ids + [mixed_id])
        mixed = srv.read(mixed_id, 64, 48, 0)
        assert srv.stats()["denoised"] >= 6
    finally:
        srv.close()
    assert np.allclose(mixed, alone, rtol=1e-6, atol=1e-7)
    # the library's own calls: halves of the frames into two films, blended
    sc = ctx.create_scene(b.desc())
    fa, fb = ctx.create_film(64, 48), ctx.create_film(64, 48)
    import copy

    ha, hb = copy.copy(shot), copy.copy(shot)
    ha.frames, hb.frame0, hb.frames = 3, 3, 3
    ctx.render(sc, ha, fa)
    ctx.render(sc, hb, fb)
    net.set_params(params)
    import torch

    with torch.cuda.stream(dn.ctx_stream(ctx)):
        want, _, _, _ = net.blended(fa, fb)
    torch.cuda.synchronize()
    assert np.allclose(want.cpu().numpy(), alone, rtol=1e-6, atol=1e-7)
