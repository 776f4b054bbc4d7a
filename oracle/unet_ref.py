"""CPU reference of the learned denoiser (test infrastructure only).

A numpy float64 restatement of the U-Net that ``asuna_gb300/csrc/denoise.cu``
runs on the GPU: the same parameter layout, padding, residual on
log1p(radiance), the training losses (L1 on log radiance, relative MSE) and
backward pass.  With ``bf16=True`` values are
rounded to bfloat16 (round to nearest even) at exactly the points where the
GPU stores bf16 tensors, so GPU and CPU differ only by accumulation order;
with ``bf16=False`` the network is plain float64 and is the one checked
against central finite differences.

The reference's own denoiser is the closed OptiX AOV denoiser
(src/tracer/denoiser.cpp:143-224); it has no restatable algorithm, so this
network is checked against itself (finite differences) and against the GPU,
not against the reference: parity unpinned.
"""
import numpy as np

IN_C = 16
HEAD_C = 16


def round_bf16(x):
    """float64 -> nearest bfloat16 value (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    bias = ((u >> 16) & 1) + 0x7FFF
    r = ((u + bias) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    return np.where(np.isfinite(f), out, f.astype(np.float64))


def layer_shapes(channels):
    """(cin, cout) of every convolution in parameter order."""
    L = len(channels)
    shapes = []
    for l in range(L):
        shapes.append((IN_C if l == 0 else channels[l - 1], channels[l]))
        shapes.append((channels[l], channels[l]))
    for l in range(L - 2, -1, -1):
        shapes.append((channels[l + 1] + channels[l], channels[l]))
        shapes.append((channels[l], channels[l]))
    shapes.append((channels[0], HEAD_C))
    return shapes


def unpack(flat, channels):
    out, off = [], 0
    for cin, cout in layer_shapes(channels):
        w = flat[off:off + cout * 9 * cin].reshape(cout, 9, cin)
        off += cout * 9 * cin
        b = flat[off:off + cout]
        off += cout
        out.append((w, b))
    assert off == flat.size
    return out


def num_params(channels):
    return sum(cout * 9 * cin + cout for cin, cout in layer_shapes(channels))


def _shift(xp, tap, h, w):
    dy, dx = tap // 3, tap % 3
    return xp[:, dy:dy + h, dx:dx + w, :]


def conv3x3(x, w, b=None):
    """x [N,H,W,Cin], w [Cout,9,Cin] -> [N,H,W,Cout]; zero padding 1."""
    n, h, wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    z = np.zeros((n, h, wd, w.shape[0]))
    for t in range(9):
        z += _shift(xp, t, h, wd) @ w[:, t, :].T
    if b is not None:
        z += b
    return z


def conv3x3_dx(dz, w):
    """Input gradient of conv3x3."""
    n, h, wd, _ = dz.shape
    dzp = np.pad(dz, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dx = np.zeros((n, h, wd, w.shape[2]))
    for t in range(9):
        dx += _shift(dzp, 8 - t, h, wd) @ w[:, t, :]
    return dx


def conv3x3_dw(dz, x):
    """Weight gradient of conv3x3: [Cout,9,Cin]."""
    n, h, wd, cin = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dzf = dz.reshape(-1, dz.shape[3])
    dw = np.zeros((dz.shape[3], 9, cin))
    for t in range(9):
        dw[:, t, :] = dzf.T @ _shift(xp, t, h, wd).reshape(-1, cin)
    return dw


def avgpool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def avgpool2_bwd(g):
    return np.repeat(np.repeat(g, 2, axis=1), 2, axis=2) * 0.25


def upsample2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample2_bwd(g):
    n, h, w, c = g.shape
    return g.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def prep_input(rad, alb, nrm, hp, wp, wsum=None, noise=None):
    """[N,H,W,4] images -> padded [N,hp,wp,16] network input (channel 9:
    log2(1 + filter-weight sum) / 16; channel 10: log1p of the mean over rgb
    of the radiance's per-pixel standard-deviation estimate, channel 11: 1
    where that estimate is given)."""
    n, h, w, _ = rad.shape
    x = np.zeros((n, hp, wp, IN_C))
    x[:, :h, :w, 0:3] = np.log1p(np.maximum(rad[..., :3], 0.0))
    if alb is not None:
        x[:, :h, :w, 3:6] = alb[..., :3]
    if nrm is not None:
        x[:, :h, :w, 6:9] = nrm[..., :3]
    if wsum is not None:
        x[:, :h, :w, 9] = np.log2(1.0 + np.maximum(wsum[..., 0], 0.0)) / 16.0
    if noise is not None:
        x[:, :h, :w, 10] = np.log1p(np.maximum(noise[..., :3].astype(np.float64).mean(axis=3), 0.0))
        x[:, :h, :w, 11] = 1.0
    return x


class UNetRef:
    """Forward / loss / backward of the denoiser in float64."""

    def __init__(self, channels, params, bf16=True):
        self.ch = list(channels)
        self.L = len(channels)
        self.layers = unpack(np.asarray(params, dtype=np.float64), self.ch)
        self.bf = bf16
        if bf16:  # the kernels read bf16 weights and fp32 biases
            self.layers = [(round_bf16(w), b) for w, b in self.layers]

    def r(self, x):
        return round_bf16(x) if self.bf else x

    def enc(self, l, k):
        return 2 * l + k

    def dec(self, l, k):
        return 2 * self.L + 2 * (self.L - 2 - l) + k

    def forward(self, rad, alb, nrm, wsum=None, noise=None):
        L = self.L
        n, h, w, _ = rad.shape
        a = 1 << (L - 1)
        hp, wp = -(-h // a) * a, -(-w // a) * a
        c = {"hp": hp, "wp": wp, "h": h, "w": w, "rad": rad}
        X = [None] * L
        A = [None] * L
        S = [None] * L
        U = [None] * L
        B = [None] * L
        D = [None] * L
        X[0] = self.r(prep_input(rad, alb, nrm, hp, wp, wsum, noise))
        for l in range(L):
            if l > 0:
                X[l] = self.r(avgpool2(S[l - 1]))
            wgt, b = self.layers[self.enc(l, 0)]
            A[l] = self.r(np.maximum(conv3x3(X[l], wgt, b), 0.0))
            wgt, b = self.layers[self.enc(l, 1)]
            S[l] = self.r(np.maximum(conv3x3(A[l], wgt, b), 0.0))
        for l in range(L - 2, -1, -1):
            src = S[L - 1] if l == L - 2 else D[l + 1]
            U[l] = np.concatenate([upsample2(src), S[l]], axis=3)
            wgt, b = self.layers[self.dec(l, 0)]
            B[l] = self.r(np.maximum(conv3x3(U[l], wgt, b), 0.0))
            wgt, b = self.layers[self.dec(l, 1)]
            D[l] = self.r(np.maximum(conv3x3(B[l], wgt, b), 0.0))
        wgt, b = self.layers[-1]
        head = conv3x3(D[0], wgt, b)
        if self.bf:
            head = head.astype(np.float32).astype(np.float64)
        c.update(X=X, A=A, S=S, U=U, B=B, D=D, head=head)
        self.cache = c
        return head

    def output(self, rad, alb, nrm, wsum=None, noise=None):
        head = self.forward(rad, alb, nrm, wsum, noise)
        n, h, w, _ = rad.shape
        y = head[:, :h, :w, :3] + np.log1p(np.maximum(rad[..., :3], 0.0))
        return np.maximum(np.expm1(y), 0.0)

    @staticmethod
    def head_loss(head3, rad, target, loss="l1log", den=None):
        """(loss, d loss / d head) of the valid head channels.  "l1log":
        mean |head + log1p(r) - log1p(t)|; "relmse": mean (o - t)^2 /
        (o + 0.01)^2 with o = max(expm1(head + log1p(r)), 0) and the
        denominator treated as a constant (or taken from `den`)."""
        count = head3.size
        y = head3 + np.log1p(np.maximum(rad[..., :3], 0.0))
        if loss == "l1log":
            d = y - np.log1p(np.maximum(target[..., :3], 0.0))
            return np.abs(d).sum() / count, np.sign(d) / count
        e = np.expm1(y)
        o = np.maximum(e, 0.0)
        inv = 1.0 / (o + 0.01) ** 2 if den is None else den
        d = o - np.maximum(target[..., :3], 0.0)
        return (d * d * inv).sum() / count, np.where(e > 0, 2.0 * d * (e + 1.0) * inv, 0.0) / count

    def loss_grad(self, rad, alb, nrm, target, wsum=None, loss="l1log", noise=None):
        """Returns (loss, flat gradient) in the parameter layout."""
        L = self.L
        head = self.forward(rad, alb, nrm, wsum, noise)
        c = self.cache
        n, h, w = rad.shape[:3]
        lv, gh = self.head_loss(head[:, :h, :w, :3], rad, target, loss)
        loss = lv
        gHead = np.zeros_like(head)
        gHead[:, :h, :w, :3] = gh
        gHead = self.r(gHead)
        grads = [None] * len(self.layers)

        def dW(li, dz, x):
            grads[li] = (conv3x3_dw(dz, x), dz.sum(axis=(0, 1, 2)))

        def dX(li, dz, mask):
            g = conv3x3_dx(dz, self.layers[li][0])
            if mask is not None:
                g = g * (mask > 0)
            return self.r(g)

        X, A, S, U, B, D = (c[k] for k in "XASUBD")
        gS = [None] * L
        gD = [None] * L
        dW(len(self.layers) - 1, gHead, D[0])
        gD[0] = dX(len(self.layers) - 1, gHead, D[0])
        for l in range(0, L - 1):
            cu = self.ch[l + 1]
            dW(self.dec(l, 1), gD[l], B[l])
            gB = dX(self.dec(l, 1), gD[l], B[l])
            dW(self.dec(l, 0), gB, U[l])
            gU = dX(self.dec(l, 0), gB, None)
            gS[l] = gU[..., cu:]
            up = self.r(upsample2_bwd(gU[..., :cu]))
            if l == L - 2:
                gS[L - 1] = up
            else:
                gD[l + 1] = up * (D[l + 1] > 0)
        for l in range(L - 1, -1, -1):
            gs = gS[l] * (S[l] > 0)
            dW(self.enc(l, 1), gs, A[l])
            gA = dX(self.enc(l, 1), gs, A[l])
            dW(self.enc(l, 0), gA, X[l])
            if l > 0:
                gX = dX(self.enc(l, 0), gA, None)
                gS[l - 1] = self.r(gS[l - 1] + avgpool2_bwd(gX))
        flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])
        return loss, flat

    def loss(self, rad, alb, nrm, target, wsum=None, loss="l1log", den=None):
        head = self.forward(rad, alb, nrm, wsum)
        n, h, w = rad.shape[:3]
        return self.head_loss(head[:, :h, :w, :3], rad, target, loss, den)[0]


def he_init(channels, seed):
    """Initial parameters of asuna_denoiser_create (splitmix64 + Box-Muller,
    He-normal weights, head scaled by 0.1, zero biases), as float32.
    splitmix64's k-th output depends only on seed + k * golden, so the draws
    are computed as one vector."""
    shapes = layer_shapes(channels)
    nw = sum(cout * 9 * cin for cin, cout in shapes)
    with np.errstate(over="ignore"):
        k = np.arange(1, 2 * nw + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    normal = np.sqrt(-2.0 * np.log(u[0::2])) * np.cos(6.283185307179586 * u[1::2])
    out, off = [], 0
    for li, (cin, cout) in enumerate(shapes):
        sd = np.sqrt(2.0 / (9.0 * cin)) * (0.1 if li == len(shapes) - 1 else 1.0)
        cnt = cout * 9 * cin
        out.append((sd * normal[off:off + cnt]).astype(np.float32))
        off += cnt
        out.append(np.zeros(cout, np.float32))
    return np.concatenate(out)
