"""Learned denoiser: Python side of include/asuna_denoise.h.

The network, its forward and backward passes and Adam run in the native
library (BF16 tensor-core kernels, FP32 accumulation).  This module holds
the thin wrapper (``Denoiser``), the training-pair generator that renders
low/high sample-count images with the library's own path tracer
(``render_pairs``), and the training loop (``train``).  Device images are
torch CUDA tensors [n, h, w, 4] float32 (torch provides the memory; every
computation is a library kernel), used on the context's stream.

Stands in for the reference's OptiX denoise step
(src/tracer/denoiser.cpp:143-224; src/tracer/tracer.cpp:531-573): radiance
with the albedo ("diffuse", multi_channel[0]) and normal (multi_channel[1])
guides.
"""
import ctypes as C
import time

import numpy as np

from . import _abi as A
from ._abi import check, lib

DEFAULT_CHANNELS = (32, 48, 64, 96, 128)
IN_CHANNELS = 16  # log1p(radiance), albedo, normal, sample count, noise, noise known, zero padding
HEAD_CHANNELS = 16  # outputs 0..2 used


def layer_table(channels=DEFAULT_CHANNELS):
    """(cin, cout, level) of every convolution in parameter order: encoder
    levels 0..L-1 (two each), decoder levels L-2..0 (two each), head."""
    L = len(channels)
    t = []
    for l in range(L):
        t += [(IN_CHANNELS if l == 0 else channels[l - 1], channels[l], l), (channels[l], channels[l], l)]
    for l in range(L - 2, -1, -1):
        t += [(channels[l + 1] + channels[l], channels[l], l), (channels[l], channels[l], l)]
    t.append((channels[0], HEAD_CHANNELS, 0))
    return t


def forward_flops(channels, hp, wp):
    """FLOPs (2 per multiply-add) of one forward pass at a padded hp x wp image."""
    return sum(2.0 * 9 * cin * cout * (hp >> l) * (wp >> l) for cin, cout, l in layer_table(channels))


def _torch():
    import torch

    return torch


def _ptr(t):
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous() and t.dtype == _torch().float32
    return C.c_void_p(t.data_ptr())


def ctx_stream(ctx):
    """The context's CUDA stream as a torch stream object."""
    torch = _torch()
    return torch.cuda.ExternalStream(lib().asuna_ctx_stream(ctx.handle))


class Denoiser:
    LOSSES = {"l1log": A.DENOISER_LOSS_L1_LOG, "relmse": A.DENOISER_LOSS_RELMSE}

    def __init__(self, ctx, channels=DEFAULT_CHANNELS, seed=0, max_pixels=1 << 20, training=False,
                 tensor_memory=True, loss="l1log"):
        self.ctx = ctx
        self.channels = tuple(int(c) for c in channels)
        o = A.DenoiserOpts()
        o.levels = len(self.channels)
        for i, c in enumerate(self.channels):
            o.channels[i] = c
        o.seed = seed
        o.max_pixels = int(max_pixels)
        o.training = 1 if training else 0
        o.tensor_memory = 1 if tensor_memory else 0
        o.loss = self.LOSSES[loss]
        h = C.c_void_p()
        check(lib().asuna_denoiser_create(ctx.handle, C.byref(o), C.byref(h)))
        self.handle = h
        self.n = int(lib().asuna_denoiser_num_params(h))
        self.align = 1 << (len(self.channels) - 1)

    # parameters --------------------------------------------------------
    def get_params(self):
        out = np.empty(self.n, np.float32)
        check(lib().asuna_denoiser_get_params(self.handle, out.ctypes.data, self.n))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().asuna_denoiser_set_params(self.handle, p.ctypes.data, p.size))

    def get_grads(self):
        out = np.empty(self.n, np.float32)
        check(lib().asuna_denoiser_get_grads(self.handle, out.ctypes.data, self.n))
        return out

    def save(self, path):
        np.savez(path, channels=np.array(self.channels), params=self.get_params())

    @classmethod
    def load(cls, ctx, path, max_pixels=1 << 22):
        z = np.load(path)
        d = cls(ctx, tuple(int(c) for c in z["channels"]), max_pixels=max_pixels)
        d.set_params(z["params"])
        return d

    # compute -----------------------------------------------------------
    def forward(self, rad, alb=None, nrm=None, wsum=None, out=None, noise=None):
        """rad/alb/nrm/wsum (film images 0, albedo, normal, 8) and the
        per-pixel noise estimate of rad (None = unknown): CUDA float32
        [n, h, w, 4]; returns the denoised radiance."""
        torch = _torch()
        n, h, w, _ = rad.shape
        if out is None:
            out = torch.empty_like(rad)
        check(lib().asuna_denoiser_forward(self.handle, _ptr(rad), _ptr(alb), _ptr(nrm), _ptr(wsum), _ptr(noise),
                                           n, h, w, _ptr(out)))
        return out

    def loss_grad(self, rad, alb, nrm, wsum, target, noise=None):
        n, h, w, _ = rad.shape
        loss = C.c_float()
        check(lib().asuna_denoiser_loss_grad(self.handle, _ptr(rad), _ptr(alb), _ptr(nrm), _ptr(wsum),
                                             _ptr(noise), _ptr(target), n, h, w, C.byref(loss)))
        return loss.value

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        check(lib().asuna_denoiser_adam(self.handle, lr, beta1, beta2, eps))

    def denoise(self, film, albedo_image=1, normal_image=2, out=None):
        """Denoises a film's radiance (image 0) into a CUDA [h, w, 4] tensor."""
        torch = _torch()
        if out is None:
            out = torch.empty((film.height, film.width, 4), dtype=torch.float32, device="cuda")
        check(lib().asuna_denoise(self.ctx.handle, self.handle, film.handle, albedo_image, normal_image, _ptr(out)))
        return out

    def estimate(self, film_a, film_b, albedo_image=1, normal_image=2, out=None):
        """Denoises film_a and estimates the RMSE of the result and of the
        plain average of both films against the converged image."""
        torch = _torch()
        if out is None:
            out = torch.empty((film_a.height, film_a.width, 4), dtype=torch.float32, device="cuda")
        ed, ep = C.c_double(), C.c_double()
        check(lib().asuna_denoise_estimate(self.ctx.handle, self.handle, film_a.handle, film_b.handle, albedo_image,
                                           normal_image, _ptr(out), C.byref(ed), C.byref(ep)))
        return out, ed.value, ep.value

    def combined(self, film_a, film_b, albedo_image=1, normal_image=2, out=None):
        """Denoises all samples of two half renders and estimates the RMSE of
        that output and of the plain average against the converged image."""
        torch = _torch()
        if out is None:
            out = torch.empty((film_a.height, film_a.width, 4), dtype=torch.float32, device="cuda")
        ed, ep = C.c_double(), C.c_double()
        check(lib().asuna_denoise_combined(self.ctx.handle, self.handle, film_a.handle, film_b.handle, albedo_image,
                                           normal_image, _ptr(out), C.byref(ed), C.byref(ep)))
        return out, ed.value, ep.value

    def blended(self, film_a, film_b, albedo_image=1, normal_image=2, out=None):
        """The all-sample denoise blended with the plain average of two half
        renders at the weight that minimises the estimated RMSE; returns
        (image, estimated RMSE, plain-average estimate, weight)."""
        torch = _torch()
        if out is None:
            out = torch.empty((film_a.height, film_a.width, 4), dtype=torch.float32, device="cuda")
        eo, ep, w = C.c_double(), C.c_double(), C.c_double()
        check(lib().asuna_denoise_blended(self.ctx.handle, self.handle, film_a.handle, film_b.handle, albedo_image,
                                          normal_image, _ptr(out), C.byref(eo), C.byref(ep), C.byref(w)))
        return out, eo.value, ep.value, w.value

    def close(self):
        if getattr(self, "handle", None):
            lib().asuna_denoiser_destroy(self.handle)
            self.handle = None

    __del__ = close


def render_pairs(ctx, seeds, width, height, spp_in=4, spp_target=256, level=4, max_depth=8):
    """Renders each training scene as two independent half renders A and B
    (own sample streams, progressive over the total counts `spp_in`: an even
    int or an increasing tuple, with the albedo / normal channels) and a
    `spp_target` render (the target).  Every (scene, count) gives two
    network inputs, as the library's blended denoise uses them: all samples
    (radiance (A + B) / 2, weight A + B, noise |A - B| / 2) and a half
    (radiance A, weight A, noise |A - B| / sqrt 2).  Returns host arrays
    [n, h, w, 4] float32: (radiance, albedo, normal, filter-weight sum,
    target, noise)."""
    from . import scenes

    levels = (spp_in,) if np.isscalar(spp_in) else tuple(spp_in)
    if any(t < 2 or t % 2 for t in levels):
        raise ValueError("sample counts must be even (two equal halves)")
    out = {k: [] for k in ("rad", "alb", "nrm", "wsum", "tgt", "noise")}
    for s in seeds:
        b, shot = scenes.training_scene(int(s), width, height, frames=levels[0], max_depth=max_depth, level=level)
        scene = ctx.create_scene(b.desc())
        g = ctx.create_film(width, height)
        shot.frame0, shot.frames, shot.seed = 0, spp_target, 3 * int(s) + 2
        ctx.render(scene, shot, g)
        tgt = g.read(0)
        fa, fb = ctx.create_film(width, height), ctx.create_film(width, height)
        done = 0
        for total in levels:
            half = total // 2
            for f, seed in ((fa, 3 * int(s)), (fb, 3 * int(s) + 1)):
                shot.frame0, shot.frames, shot.seed = done, half - done, seed
                ctx.render(scene, shot, f)
            done = half
            a, bb = fa.read(0), fb.read(0)
            wa, wb = fa.read(8), fb.read(8)
            alb, nrm = fa.read(1), fa.read(2)
            diff = np.abs(a - bb)
            allr = 0.5 * (a + bb)
            allr[..., 3] = 1.0
            for rad, wsum, noise in ((allr, wa + wb, diff * np.float32(0.5)),
                                     (a, wa, diff * np.float32(0.70710678))):
                out["rad"].append(rad)
                out["alb"].append(alb)
                out["nrm"].append(nrm)
                out["wsum"].append(wsum)
                out["tgt"].append(tgt)
                out["noise"].append(noise)
        fa.close()
        fb.close()
        g.close()
        del scene
    return tuple(np.stack(out[k]) for k in ("rad", "alb", "nrm", "wsum", "tgt", "noise"))


def train(den, data, steps, batch=8, crop=64, lr=1e-3, seed=0, log_every=0):
    """Adam on random crops of the training pairs.  `data` = (rad, alb, nrm,
    wsum, tgt[, noise]) host arrays [n, h, w, 4]; returns the loss history."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in data]
    torch.cuda.synchronize()
    n, h, w, _ = data[0].shape
    losses = []
    t0 = time.perf_counter()
    with torch.cuda.stream(ctx_stream(den.ctx)):
        for it in range(steps):
            idx = rng.integers(0, n, batch)
            ys = rng.integers(0, h - crop + 1, batch)
            xs = rng.integers(0, w - crop + 1, batch)
            crops = [torch.stack([a[int(idx[k]), ys[k]:ys[k] + crop, xs[k]:xs[k] + crop] for k in range(batch)])
                     .contiguous() for a in dev]
            loss = den.loss_grad(*crops[:5], noise=crops[5] if len(crops) > 5 else None)
            den.adam(lr)
            losses.append(loss)
            if log_every and (it + 1) % log_every == 0:
                print(f"step {it + 1}: loss {np.mean(losses[-log_every:]):.4f} "
                      f"({time.perf_counter() - t0:.1f} s)", flush=True)
    den.ctx.sync()
    return losses


def rmse(a, b):
    a = np.asarray(a, np.float64)[..., :3]
    b = np.asarray(b, np.float64)[..., :3]
    return float(np.sqrt(np.mean((a - b) ** 2)))
