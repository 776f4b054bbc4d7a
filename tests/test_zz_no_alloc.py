"""asuna_render_noalloc: the render entry point for callers that cannot
allocate device memory while they render (a memory pool or budget held by its
owner, a fixed footprint granted up front, a render thread kept out of the
allocator).  Its scratch lives in one fixed array compiled into the library.

Checked through the C ABI against asuna_render on two calls in a row (the
second call starts from the array the first one left behind), within the
tolerance of the other GPU tests (identical kernels, so the films agree to
float rounding of the same operations); on shots that take several batches
of the fixed path slots (3 and 65 batches); the size limit is enforced, a
traversal cut short is reported, and a capturing stream is refused.
Collected last so that a failure here leaves every other test already run;
it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import asuna_gb300 as ag
from asuna_gb300 import _abi as A
from asuna_gb300 import scenes

pytestmark = pytest.mark.gpu


def _noalloc():
    fn = A.lib().asuna_render_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.POINTER(A.Shot), C.c_void_p, C.c_void_p]
    return fn


def _films(film):
    return np.stack([film.read(k) for k in range(A.NUM_OUTPUT_IMAGES)])


def _expect(ctx, scene, shot):
    f = ctx.create_film(shot.width, shot.height)
    ctx.render(scene, shot, f)
    out = _films(f)
    f.close()
    return out


def _close(a, b):
    # same bound as the GPU parity tests: 1e-4 relative, 1e-6 absolute
    return np.all(np.abs(a - b) <= 1e-4 * np.abs(b) + 1e-6)


def test_noalloc_matches_render_on_two_calls_in_a_row():
    ctx = ag.Context(0)
    fn = _noalloc()
    b1, s1 = scenes.plugin_scene(96, 64, frames=3, max_depth=6)
    b2, s2 = scenes.box_scene(80, 72, frames=5, max_depth=8)
    sc1, sc2 = ctx.create_scene(b1.desc()), ctx.create_scene(b2.desc())
    want1, want2 = _expect(ctx, sc1, s1), _expect(ctx, sc2, s2)
    f1, f2 = ctx.create_film(s1.width, s1.height), ctx.create_film(s2.width, s2.height)
    stream = A.lib().asuna_ctx_stream(ctx.handle)  # film reads are ordered on this stream
    A.check(fn(sc1.handle, C.byref(s1), f1.handle, stream))
    A.check(fn(sc2.handle, C.byref(s2), f2.handle, stream))
    got1, got2 = _films(f1), _films(f2)
    assert _close(got1, want1) and _close(got2, want2)
    assert float(got2[0, ..., :3].mean()) > 0.0


def test_noalloc_rejects_frames_beyond_its_scratch():
    ctx = ag.Context(0)
    fn = _noalloc()
    b, s = scenes.box_scene(8, 8, frames=1, max_depth=2)
    scene = ctx.create_scene(b.desc())
    side = 513  # 513 x 513 pixels > ASUNA_NOALLOC_MAX_PATHS (262,144)
    s.width = s.height = side
    film = ctx.create_film(side, side)
    rc = fn(scene.handle, C.byref(s), film.handle, None)
    assert rc == A.ERR_INVALID
    assert b"exceeds the scratch maximum" in A.lib().asuna_last_error()


@pytest.mark.parametrize("width,height,frames", [(512, 512, 3), (512, 256, 129)])
def test_noalloc_matches_render_over_many_batches(width, height, frames):
    """512 x 512 takes one frame per batch (3 batches); 512 x 256 two frames
    per batch (65 batches), each reusing the same path slots."""
    ctx = ag.Context(0)
    fn = _noalloc()
    b, s = scenes.box_scene(width, height, frames=frames, max_depth=3)
    sc = ctx.create_scene(b.desc())
    want = _expect(ctx, sc, s)
    f = ctx.create_film(width, height)
    stream = A.lib().asuna_ctx_stream(ctx.handle)
    A.check(fn(sc.handle, C.byref(s), f.handle, stream))
    got = _films(f)
    assert _close(got, want)
    assert float(got[8, ..., 0].min()) > 0.0  # every pixel has its filter weight


def test_noalloc_reports_a_runaway_traversal_and_recovers():
    """70,000 coincident instances drive every camera ray into the
    traversal's loop bound: the call returns ERR_TRAVERSAL.  The next call
    starts from a cleared count and succeeds."""
    ctx = ag.Context(0)
    fn = _noalloc()
    b, s = scenes.stacked_instances_scene(70000)
    sc = ctx.create_scene(b.desc())
    f = ctx.create_film(s.width, s.height)
    rc = fn(sc.handle, C.byref(s), f.handle, None)
    assert rc == A.ERR_TRAVERSAL
    assert b"cut short" in A.lib().asuna_last_error()
    b2, s2 = scenes.box_scene(16, 16, frames=1, max_depth=2)
    sc2 = ctx.create_scene(b2.desc())
    f2 = ctx.create_film(16, 16)
    A.check(fn(sc2.handle, C.byref(s2), f2.handle, None))


def test_noalloc_refuses_a_capturing_stream():
    """The call waits for its work, so on a stream being captured it queues
    nothing and returns ERR_UNSUPPORTED; the capture itself stays valid."""
    import torch

    ctx = ag.Context(0)
    fn = _noalloc()
    b, s = scenes.box_scene(16, 16, frames=1, max_depth=2)
    sc = ctx.create_scene(b.desc())
    f = ctx.create_film(16, 16)
    A.check(fn(sc.handle, C.byref(s), f.handle, None))  # set-up on this device happens outside the capture
    x = torch.zeros(4, device="cuda:0")
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    with torch.cuda.graph(g, stream=side):
        rc = fn(sc.handle, C.byref(s), f.handle, C.c_void_p(side.cuda_stream))
        x.add_(1.0)
    assert rc == A.ERR_UNSUPPORTED
    g.replay()
    torch.cuda.synchronize()
    assert float(x.sum()) == 4.0
