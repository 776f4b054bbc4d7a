"""CPU reference of the denoiser: its backward pass agrees with float64
central finite differences, bf16 rounding is round-to-nearest-even, and the
initial parameters follow the library's seeded He-normal recipe."""
import numpy as np
import pytest

from oracle import unet_ref as U


def _images(rng, n, h, w):
    rad = rng.gamma(1.5, 0.4, (n, h, w, 4))
    alb = rng.uniform(0.0, 1.0, (n, h, w, 4))
    nrm = rng.normal(size=(n, h, w, 4))
    tgt = rad * rng.uniform(0.6, 1.4, rad.shape)
    return rad, alb, nrm, tgt


def test_sample_count_channel():
    rad = np.ones((1, 4, 4, 4))
    w = np.full((1, 4, 4, 4), 255.0)
    x = U.prep_input(rad, None, None, 16, 16, w)
    assert np.allclose(x[0, :4, :4, 9], 0.5) and not x[0, 4:, :, 9].any()


@pytest.mark.parametrize("loss_kind", ["l1log", "relmse"])
def test_backward_matches_finite_differences(loss_kind):
    """Central differences of the float64 network; relmse's denominator is
    held at the unperturbed output, as the gradient treats it."""
    rng = np.random.default_rng(3)
    ch = [4, 6, 8]
    params = U.he_init(ch, 5).astype(np.float64)
    params += rng.normal(0, 0.05, params.size)  # non-zero biases too
    rad, alb, nrm, tgt = _images(rng, 2, 7, 9)  # padded to 8 x 12
    net = U.UNetRef(ch, params, bf16=False)
    loss, g = net.loss_grad(rad, alb, nrm, tgt, loss=loss_kind)
    den = None
    if loss_kind == "relmse":
        den = 1.0 / (net.output(rad, alb, nrm)[..., :3] + 0.01) ** 2
    assert np.isclose(loss, net.loss(rad, alb, nrm, tgt, loss=loss_kind, den=den))
    # central differences on the largest-gradient parameters of every layer
    off, picks = 0, []
    for cin, cout in U.layer_shapes(ch):
        n = cout * 9 * cin + cout
        seg = np.abs(g[off:off + n])
        picks += list(off + np.argsort(seg)[-3:])
        off += n
    eps = 1e-6
    for i in picks:
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        fd = (U.UNetRef(ch, p1, bf16=False).loss(rad, alb, nrm, tgt, loss=loss_kind, den=den) -
              U.UNetRef(ch, p2, bf16=False).loss(rad, alb, nrm, tgt, loss=loss_kind, den=den)) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-7 + 2e-4 * abs(fd), (i, fd, g[i])


def test_conv_gradients_are_adjoint():
    # <conv(x), dz> = <x, conv_dx(dz)> = <w, conv_dw(dz, x)>
    rng = np.random.default_rng(1)
    x = rng.normal(size=(2, 5, 6, 3))
    w = rng.normal(size=(4, 9, 3))
    dz = rng.normal(size=(2, 5, 6, 4))
    z = U.conv3x3(x, w)
    a = np.sum(z * dz)
    assert np.isclose(a, np.sum(x * U.conv3x3_dx(dz, w)))
    assert np.isclose(a, np.sum(w * U.conv3x3_dw(dz, x)))


def test_round_bf16():
    v = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -3.14159, 0.0, 1e-40, 65504.0])
    r = U.round_bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0  # tie -> even
    assert r[2] == 1.0078125  # above the tie
    assert r[3] == 1.0078125
    assert r[4] == -3.140625
    assert r[5] == 0.0
    assert np.all(U.round_bf16(r) == r)


def test_init_layout_and_scale():
    ch = [32, 48, 64, 96, 128]
    p = U.he_init(ch, 11)
    assert p.size == U.num_params(ch) == 1021904
    layers = U.unpack(p.astype(np.float64), ch)
    assert len(layers) == 4 * len(ch) - 1
    for (w, b), (cin, cout) in zip(layers[:-1], U.layer_shapes(ch)[:-1]):
        assert np.all(b == 0)
        assert abs(w.std() / np.sqrt(2.0 / (9 * cin)) - 1.0) < 0.1
    assert np.array_equal(p, U.he_init(ch, 11))
    assert not np.array_equal(p, U.he_init(ch, 12))


def test_package_layer_table_matches_reference():
    from asuna_gb300 import denoise as dn

    ch = dn.DEFAULT_CHANNELS
    assert [(a, b) for a, b, _ in dn.layer_table(ch)] == U.layer_shapes(list(ch))
    # 0.40 TFLOP per forward of a padded 1088 x 1920 image
    assert abs(dn.forward_flops(ch, 1088, 1920) / 1e12 - 0.4019) < 1e-3
