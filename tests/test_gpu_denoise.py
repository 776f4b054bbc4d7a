"""Denoiser kernels on the GPU against the CPU reference (oracle/unet_ref.py):
each BF16 tensor-core kernel, then the whole network's forward output, loss
and parameter gradients; then training on renderer-made pairs and what the
trained network gains over the noisy input."""
import ctypes as C

import numpy as np
import pytest

import asuna_gb300 as ag
from asuna_gb300 import _abi as A
from asuna_gb300 import denoise as dn
from oracle import unet_ref as U

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def bf16(a):
    return torch.from_numpy(np.asarray(a, np.float32)).cuda().to(torch.bfloat16).contiguous()


def f32(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.float().cpu().numpy().astype(np.float64)


def ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


@pytest.fixture(scope="module")
def lib():
    return A.lib()


@pytest.fixture(scope="module")
def dctx():
    return ag.Context(0)


def run(lib, name, *args):
    A.check(getattr(lib, name)(None, *args))  # default stream: ordered with torch's own work
    torch.cuda.synchronize()


@pytest.mark.parametrize("shape", [(2, 20, 24, 32, 48), (1, 9, 13, 16, 8), (1, 33, 70, 224, 96)])
def test_conv3x3_forward(lib, shape):
    n, h, w, cin, cout = shape
    rng = np.random.default_rng(cin + cout)
    x = U.round_bf16(rng.normal(size=(n, h, w, cin)))
    wt = U.round_bf16(rng.normal(0, 0.2, (cout, 9, cin)))
    b = rng.normal(0, 0.1, cout).astype(np.float32)
    ref = U.conv3x3(x, wt, b.astype(np.float64))
    dx, dwt, db = bf16(x), bf16(wt), f32(b)  # named: alive until the kernels ran
    out = torch.empty((n, h, w, cout), dtype=torch.float32, device="cuda")
    run(lib, "asuna_nn_conv3x3", ptr(dx), n, h, w, cin, ptr(dwt), ptr(db), cout, 0, None, ptr(out), 1)
    got = host(out)
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 2e-5 * scale
    # bf16 output with ReLU: equal to the rounded reference up to one bf16 step
    outb = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    run(lib, "asuna_nn_conv3x3", ptr(dx), n, h, w, cin, ptr(dwt), ptr(db), cout, 1, None, ptr(outb), 0)
    gb = host(outb)
    rr = U.round_bf16(np.maximum(ref, 0))
    # one bf16 step, plus the fp32 accumulation error near the ReLU kink
    assert np.all(np.abs(gb - rr) <= np.abs(rr) * 2.0 ** -7 + 2e-5 * scale)
    assert np.mean(gb == rr) > 0.98


def test_conv3x3_input_gradient_with_mask(lib):
    n, h, w, cin, cout = 2, 17, 30, 48, 32
    rng = np.random.default_rng(7)
    dz = U.round_bf16(rng.normal(size=(n, h, w, cout)))
    wt = U.round_bf16(rng.normal(0, 0.2, (cout, 9, cin)))
    mask = U.round_bf16(rng.normal(size=(n, h, w, cin)))
    ddz, dwt, dmask = bf16(dz), bf16(wt), bf16(mask)
    wflip = torch.empty((cin, 9, cout), dtype=torch.bfloat16, device="cuda")
    run(lib, "asuna_nn_flip_weights", ptr(dwt), ptr(wflip), cout, cin)
    assert np.array_equal(host(wflip), wt.transpose(2, 1, 0)[:, ::-1, :])
    out = torch.empty((n, h, w, cin), dtype=torch.float32, device="cuda")
    run(lib, "asuna_nn_conv3x3", ptr(ddz), n, h, w, cout, ptr(wflip), None, cin, 0, ptr(dmask), ptr(out), 1)
    ref = U.conv3x3_dx(dz, wt) * (mask > 0)
    assert np.abs(host(out) - ref).max() <= 2e-5 * np.abs(ref).max()


@pytest.mark.parametrize("shape", [(1, 16, 8, 16, 16), (2, 20, 24, 32, 48), (1, 33, 70, 224, 96),
                                   (1, 40, 37, 48, 128), (3, 9, 13, 16, 32), (1, 24, 16, 96, 64),
                                   (1, 20, 30, 32, 224), (2, 12, 20, 16, 256), (1, 17, 19, 48, 192)])
def test_conv3x3_tcgen05(lib, shape):
    """The tcgen05 / TMEM / TMA convolution against the float64 reference:
    edge tiles (sizes not multiples of 16 x 8), batches, 16..224 input and
    16..256 output channels (192, 224 and 256 split over two CTAs per tile);
    bias, ReLU, mask and fp32 / bf16 outputs."""
    n, h, w, cin, cout = shape
    rng = np.random.default_rng(cin * 7 + cout)
    x = U.round_bf16(rng.normal(size=(n, h, w, cin)))
    wt = U.round_bf16(rng.normal(0, 0.2, (cout, 9, cin)))
    b = rng.normal(0, 0.1, cout).astype(np.float32)
    mask = U.round_bf16(rng.normal(size=(n, h, w, cout)))
    dx, dwt, db, dmask = bf16(x), bf16(wt), f32(b), bf16(mask)
    wtc = torch.empty(cout * 9 * cin, dtype=torch.bfloat16, device="cuda")
    run(lib, "asuna_nn_weights_tc", ptr(dwt), ptr(wtc), cout, cin)
    out = torch.full((n, h, w, cout), float("nan"), dtype=torch.float32, device="cuda")
    run(lib, "asuna_nn_conv3x3_tc", ptr(dx), n, h, w, cin, ptr(wtc), ptr(db), cout, 0, None, ptr(out), 1)
    expired = C.c_int(-1)
    A.check(lib.asuna_nn_tc_status(C.byref(expired)))
    assert expired.value == 0
    ref = U.conv3x3(x, wt, b.astype(np.float64))
    got = host(out)
    assert np.isfinite(got).all()
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()
    outb = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    run(lib, "asuna_nn_conv3x3_tc", ptr(dx), n, h, w, cin, ptr(wtc), ptr(db), cout, 1, ptr(dmask), ptr(outb), 0)
    rr = U.round_bf16(np.maximum(ref, 0) * (mask > 0))
    gb = host(outb)
    assert np.all(np.abs(gb - rr) <= np.abs(rr) * 2.0 ** -7 + 2e-5 * np.abs(ref).max())
    A.check(lib.asuna_nn_tc_status(C.byref(expired)))
    assert expired.value == 0


def test_network_on_tcgen05_matches_mma_sync(dctx):
    """The whole denoiser (forward, loss, gradients) with every forward and
    input-gradient convolution on tcgen05 equals the mma.sync network up to
    accumulation order."""
    rng = np.random.default_rng(8)
    n, h, w = 2, 40, 56
    rad, alb, nrm, wsum, tgt = _net_inputs(rng, n, h, w)
    p = U.he_init(dn.DEFAULT_CHANNELS, 4)
    p = (p + rng.normal(0, 0.02, p.size)).astype(np.float32)
    res = []
    for tm in (False, True):
        d = dn.Denoiser(dctx, seed=4, max_pixels=n * 48 * 64, training=True, tensor_memory=tm)
        d.set_params(p)
        drad, dalb, dnrm, dw, dtgt = f32(rad), f32(alb), f32(nrm), f32(wsum), f32(tgt)
        torch.cuda.synchronize()
        out = d.forward(drad, dalb, dnrm, dw)
        dctx.sync()
        loss = d.loss_grad(drad, dalb, dnrm, dw, dtgt)
        res.append((out.cpu().numpy(), loss, d.get_grads().astype(np.float64)))
    (o0, l0, g0), (o1, l1, g1) = res
    assert np.median(np.abs(o1 - o0) / (np.abs(o0) + 1e-3)) < 2e-3
    assert abs(l1 - l0) <= 1e-3 * l0
    rel = np.linalg.norm(g1 - g0) / np.linalg.norm(g0)
    assert rel < 0.03, rel


@pytest.mark.parametrize("shape", [(2, 40, 64, 32, 48), (1, 16, 16, 16, 16), (3, 23, 37, 112, 48)])
def test_conv3x3_weight_gradient(lib, shape):
    n, h, w, cin, cout = shape  # > 2048 pixels: several split-K blocks
    rng = np.random.default_rng(cin * 3 + cout)
    x = U.round_bf16(rng.normal(size=(n, h, w, cin)))
    dz = U.round_bf16(rng.normal(size=(n, h, w, cout)))
    ddz, dx = bf16(dz), bf16(x)
    dw = torch.zeros((cout, 9, cin), dtype=torch.float32, device="cuda")
    run(lib, "asuna_nn_conv3x3_wgrad", ptr(ddz), ptr(dx), n, h, w, cin, cout, ptr(dw))
    ref = U.conv3x3_dw(dz, x)
    assert np.abs(host(dw) - ref).max() <= 2e-5 * np.abs(ref).max()
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    run(lib, "asuna_nn_bias_grad", ptr(ddz), n * h * w, cout, ptr(db))
    assert np.allclose(host(db), dz.sum(axis=(0, 1, 2)), rtol=1e-5, atol=1e-3)


def test_pool_upsample_copy_and_mask(lib):
    n, h, w, c = 2, 12, 20, 32
    rng = np.random.default_rng(2)
    x = U.round_bf16(rng.normal(size=(n, h, w, c)))
    dx = bf16(x)
    out = torch.empty((n, h // 2, w // 2, c), dtype=torch.bfloat16, device="cuda")
    run(lib, "asuna_nn_avgpool2", ptr(dx), ptr(out), n, h, w, c)
    assert np.abs(host(out) - U.round_bf16(U.avgpool2(x))).max() <= 2.0 ** -7 * np.abs(x).max()
    g = U.round_bf16(rng.normal(size=(n, h // 2, w // 2, c)))
    din, dg = bf16(x), bf16(g)
    run(lib, "asuna_nn_avgpool2_bwd", ptr(dg), ptr(din), n, h, w, c, 1)
    ref = U.round_bf16(x + U.avgpool2_bwd(g))
    assert np.abs(host(din) - ref).max() <= 2.0 ** -7 * np.abs(ref).max()
    # nearest x2 into channels [8, 8 + c) of a 48-channel buffer, and back
    small = U.round_bf16(rng.normal(size=(n, h // 2, w // 2, c)))
    dsmall = bf16(small)
    big = torch.zeros((n, h, w, 48), dtype=torch.bfloat16, device="cuda")
    run(lib, "asuna_nn_upsample2", ptr(dsmall), ptr(big), n, h, w, c, 48, 8)
    hb = host(big)
    assert np.array_equal(hb[..., 8:8 + c], U.upsample2(small)) and not hb[..., :8].any()
    back = torch.empty((n, h // 2, w // 2, c), dtype=torch.bfloat16, device="cuda")
    run(lib, "asuna_nn_upsample2_bwd", ptr(big), ptr(back), n, h // 2, w // 2, c, 48, 8)
    assert np.array_equal(host(back), U.round_bf16(4 * small))
    dst = torch.zeros((n, h, w, 16), dtype=torch.bfloat16, device="cuda")
    run(lib, "asuna_nn_copy_channels", ptr(big), 48, 10, ptr(dst), 16, 4, 8, n * h * w, 0)
    assert np.array_equal(host(dst)[..., 4:12], hb[..., 10:18])
    # 8-channel-aligned offsets take the 16-byte kernels; accumulate adds in fp32
    run(lib, "asuna_nn_copy_channels", ptr(big), 48, 8, ptr(dst), 16, 8, 8, n * h * w, 1)
    want = host(dst)
    assert np.array_equal(want[..., 8:12], U.round_bf16(hb[..., 14:18] + hb[..., 8:12]))
    assert np.array_equal(want[..., 12:16], hb[..., 12:16]) and np.array_equal(want[..., 4:8], hb[..., 10:14])
    # channel counts that are not multiples of 8 take the per-element kernels
    x12 = U.round_bf16(rng.normal(size=(n, h, w, 12)))
    o12 = torch.empty((n, h // 2, w // 2, 12), dtype=torch.bfloat16, device="cuda")
    d12 = bf16(x12)
    run(lib, "asuna_nn_avgpool2", ptr(d12), ptr(o12), n, h, w, 12)
    assert np.abs(host(o12) - U.round_bf16(U.avgpool2(x12))).max() <= 2.0 ** -7 * np.abs(x12).max()
    m = bf16(x)
    y = U.round_bf16(rng.normal(size=x.shape))
    dy = bf16(y)
    run(lib, "asuna_nn_relu_mask", ptr(m), ptr(dy), x.size)
    assert np.array_equal(host(m), x * (y > 0))


def _net_inputs(rng, n, h, w):
    rad = rng.gamma(1.2, 0.5, (n, h, w, 4)).astype(np.float32)
    alb = rng.uniform(0, 1, (n, h, w, 4)).astype(np.float32)
    nrm = rng.normal(size=(n, h, w, 4)).astype(np.float32)
    wsum = np.repeat(rng.uniform(1.0, 600.0, (n, h, w, 1)), 4, axis=3).astype(np.float32)
    tgt = (rad * rng.uniform(0.5, 1.5, rad.shape)).astype(np.float32)
    return rad, alb, nrm, wsum, tgt


@pytest.mark.parametrize("loss_kind,with_noise", [("l1log", False), ("relmse", False), ("l1log", True)])
def test_network_forward_loss_and_gradients(dctx, loss_kind, with_noise):
    ch = dn.DEFAULT_CHANNELS
    rng = np.random.default_rng(5)
    n, h, w = 2, 37, 45  # padded to 48 x 48
    rad, alb, nrm, wsum, tgt = _net_inputs(rng, n, h, w)
    noise = rng.uniform(0.0, 2.0, rad.shape).astype(np.float32) if with_noise else None
    d = dn.Denoiser(dctx, ch, seed=3, max_pixels=n * 48 * 48, training=True, loss=loss_kind)
    p = U.he_init(ch, 3)
    assert np.allclose(d.get_params(), p, rtol=1e-6, atol=1e-9)
    p = (p + rng.normal(0, 0.02, p.size)).astype(np.float32)  # non-zero biases, active head
    d.set_params(p)
    ref = U.UNetRef(ch, p, bf16=True)
    drad, dalb, dnrm, dw, dtgt = f32(rad), f32(alb), f32(nrm), f32(wsum), f32(tgt)
    dnoise = f32(noise) if with_noise else None
    torch.cuda.synchronize()
    out = d.forward(drad, dalb, dnrm, dw, noise=dnoise)
    dctx.sync()
    ro = ref.output(rad.astype(np.float64), alb, nrm, wsum, noise)
    got = out.cpu().numpy()[..., :3]
    med = np.median(np.abs(got - ro) / (np.abs(ro) + 1e-3))
    mx = np.abs(got - ro).max() / np.abs(ro).max()
    loss = d.loss_grad(drad, dalb, dnrm, dw, dtgt, noise=dnoise)
    rl, rg = ref.loss_grad(rad.astype(np.float64), alb, nrm, tgt.astype(np.float64), wsum, loss=loss_kind,
                           noise=noise)
    g = d.get_grads().astype(np.float64)
    print(f"\nforward: median rel {med:.2e}, max/scale {mx:.2e}; loss {loss:.6f} vs {rl:.6f}")
    off, rows = 0, []
    for li, (cin, cout) in enumerate(U.layer_shapes(list(ch))):
        k = cout * 9 * cin + cout
        a, b = g[off:off + k], rg[off:off + k]
        off += k
        if not np.any(b):
            continue
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
        rows.append((li, rel, cos))
        print(f"layer {li:2d} ({cin:3d}->{cout:3d}): grad rel err {rel:.2e}, cosine {cos:.6f}")
    # tolerances: accumulation order only (the reference rounds to bf16 where the kernels store bf16);
    # relmse weights each pixel by 1 / (out + 0.01)^2, up to 10^4 where the output is near 0, which
    # magnifies those differences in the deepest layers
    assert med < 5e-3 and mx < 0.05
    assert abs(loss - rl) <= 2e-3 * rl
    rel_max, cos_min = (0.05, 0.998) if loss_kind == "l1log" else (0.2, 0.99)
    for li, rel, cos in rows:
        assert rel < rel_max and cos > cos_min, (li, rel, cos)


def test_training_gain_over_noisy_input(dctx):
    """Train on 4-spp / 256-spp pairs of 24 seeded scenes (two 2-spp halves
    each, as all samples and as a half, with their per-pixel noise); on 4
    held-out scenes the denoised input is much closer to the 256-spp render
    than the input is."""
    train = dn.render_pairs(dctx, range(24), 96, 96, spp_in=4, spp_target=256, level=3)
    test = dn.render_pairs(dctx, range(100, 104), 96, 96, spp_in=4, spp_target=256, level=3)
    d = dn.Denoiser(dctx, seed=1, max_pixels=8 * 64 * 64, training=True)
    losses = dn.train(d, train, steps=400, batch=8, crop=64, lr=1e-3)
    assert np.mean(losses[-50:]) < 0.8 * np.mean(losses[:10])
    e = dn.Denoiser(dctx, max_pixels=8 * 96 * 96)
    e.set_params(d.get_params())
    rad, alb, nrm, wsum, tgt, noise = test
    drad, dalb, dnrm, dw = f32(rad), f32(alb), f32(nrm), f32(wsum)
    torch.cuda.synchronize()
    out = e.forward(drad, dalb, dnrm, dw, noise=f32(noise))
    dctx.sync()
    den = out.cpu().numpy()
    noisy_err = dn.rmse(rad, tgt)
    den_err = dn.rmse(den, tgt)
    print(f"held-out RMSE vs 256 spp: noisy {noisy_err:.4f}, denoised {den_err:.4f}")
    assert den_err < 0.7 * noisy_err


def test_film_denoise_and_error_estimate(dctx):
    from asuna_gb300 import scenes

    b, shot = scenes.training_scene(7, 80, 64, frames=8, level=3)
    scene = dctx.create_scene(b.desc())
    fa, fb = dctx.create_film(80, 64), dctx.create_film(80, 64)
    shot.frame0 = 0
    dctx.render(scene, shot, fa)
    shot.frame0 = 8
    dctx.render(scene, shot, fb)
    d = dn.Denoiser(dctx, seed=2, max_pixels=80 * 64)
    out = d.denoise(fa)
    dctx.sync()
    # the untrained head is small: the output stays close to the input radiance
    a = fa.read(0)
    assert np.isfinite(out.cpu().numpy()).all()
    assert dn.rmse(out.cpu().numpy(), a) < 0.5 * np.sqrt(np.mean(a[..., :3] ** 2)) + 1e-3
    den, ed, ep = d.estimate(fa, fb)
    dctx.sync()
    bb = fb.read(0)
    mab = np.mean((a[..., :3].astype(np.float64) - bb[..., :3]) ** 2)
    assert np.isclose(ep, np.sqrt(mab / 4), rtol=1e-4)
    mdb = np.mean((den.cpu().numpy()[..., :3].astype(np.float64) - bb[..., :3]) ** 2)
    assert np.isclose(ed, np.sqrt(max(0.0, mdb - mab / 2)), rtol=1e-3, atol=1e-6)
    # all samples: the output is the denoiser on (A + B) / 2 with weight A + B;
    # the estimate subtracts half the halves' output variance
    full, ec, ep2 = d.combined(fa, fb)
    dctx.sync()
    import torch

    # the per-pixel noise the two halves give: |a - b| / sqrt(2) for a half,
    # |a - b| / 2 for their average
    diff = np.abs(a - bb).astype(np.float32)
    n_half, n_all = torch.from_numpy(diff * np.float32(0.70710678))[None].cuda(), \
        torch.from_numpy(diff * np.float32(0.5))[None].cuda()
    db_ = d.forward(fb.tensor(0)[None].contiguous(), fb.tensor(1)[None].contiguous(), fb.tensor(2)[None].contiguous(),
                    fb.tensor(8)[None].contiguous(), noise=n_half)
    dctx.sync()  # the library's stream, not torch's: wait before the copy
    db_ = db_[0].cpu().numpy()
    comb = 0.5 * (a + bb)
    comb[..., 3] = 1.0
    ref = d.forward(torch.from_numpy(comb)[None].cuda(), fa.tensor(1)[None].contiguous(),
                    fa.tensor(2)[None].contiguous(), (fa.tensor(8) + fb.tensor(8))[None], noise=n_all)
    dctx.sync()
    assert np.allclose(full.cpu().numpy(), ref[0].cpu().numpy(), atol=1e-6)
    var_half = 0.5 * np.mean((den.cpu().numpy()[..., :3].astype(np.float64) - db_[..., :3]) ** 2)
    assert np.isclose(ec, np.sqrt(max(0.0, ed * ed - 0.5 * var_half)), rtol=1e-3, atol=1e-6)
    assert ep2 == pytest.approx(ep)
    # the blend of that output with the plain average, at the weight that
    # minimises the estimate (a quadratic in w)
    bl, eo, ep3, wgt = d.blended(fa, fb)
    dctx.sync()
    assert 0.0 <= wgt <= 1.0 and ep3 == pytest.approx(ep)
    plain = 0.5 * (a + bb)
    want = wgt * full.cpu().numpy()[..., :3] + (1.0 - wgt) * plain[..., :3]
    assert np.allclose(bl.cpu().numpy()[..., :3], want, rtol=1e-5, atol=1e-5)
    da_, db2 = den.cpu().numpy()[..., :3].astype(np.float64), db_[..., :3]
    a3, b3 = a[..., :3].astype(np.float64), bb[..., :3].astype(np.float64)

    def est(w):
        xa, xb = w * da_ + (1 - w) * a3, w * db2 + (1 - w) * b3
        return np.mean((xa - b3) ** 2) - np.mean((a3 - b3) ** 2) / 2 - np.mean((xa - xb) ** 2) / 4

    assert np.isclose(eo, np.sqrt(max(0.0, est(wgt))), rtol=1e-3, atol=1e-6)
    assert all(est(wgt) <= est(w) + 1e-3 * est(0.0) for w in np.linspace(0, 1, 21))
    assert eo <= min(ec, ep) * (1 + 1e-6)
    with pytest.raises(A.AsunaError):
        d.denoise(fa, albedo_image=0)
    big = dctx.create_film(256, 256)
    with pytest.raises(A.AsunaError):
        d.denoise(big)  # larger than max_pixels: rejected, not overrun
    with pytest.raises(A.AsunaError):
        d.combined(fa, big)  # the halves must have one size
    with pytest.raises(A.AsunaError):
        d.blended(big, fb)
