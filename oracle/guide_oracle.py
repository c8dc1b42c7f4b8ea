"""CPU oracle of the learned guiding proposal: the 9 -> 64 -> 64 -> 64 -> 40 MLP, the
8-lobe von Mises-Fisher mixture, its training loss and gradient, written from the math
in numpy (float64), with the device's BF16 rounding of weights and activations
emulated.  TEST INFRASTRUCTURE ONLY (the network has no counterpart in the reference
renderer).

Parameter layout (as spgpu_guiding_params): each layer's weights [out][in] row-major,
then its bias: W1 64x9, b1, W2 64x64, b2, W3 64x64, b3, W4 40x64, b4 -> 11,560 floats.
Raw output j of lobe k: 5k+0..2 unnormalised axis, 5k+3 log-concentration (clamped to
[-4, 7]), 5k+4 weight logit (softmax).
vMF density: kappa / (2 pi (1 - exp(-2 kappa))) * exp(kappa (mu . w - 1)).
Loss over a batch: sum_i c_i (-log q(w_i)) / sum_i c_i.
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT, LOBES = 9, 64, 40, 8
SHAPES = [(HID, IN), (HID, HID), (HID, HID), (OUT, HID)]
N_PARAMS = sum(o * i + o for o, i in SHAPES)


def unpack(p):
    p = np.asarray(p, np.float64)
    layers, off = [], 0
    for o, i in SHAPES:
        W = p[off:off + o * i].reshape(o, i)
        off += o * i
        b = p[off:off + o]
        off += o
        layers.append((W, b))
    return layers


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, np.float32).copy()
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(p, x, emulate_bf16=True):
    """Raw outputs (n, 40) and the hidden activations (post-ReLU, as the device stores them)."""
    q = bf16 if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    L = unpack(p)
    h = q(x)
    acts = [h]
    for li, (W, b) in enumerate(L):
        z = h @ q(W).T + b
        if li < 3:
            h = q(np.maximum(z, 0.0))
            acts.append(h)
        else:
            h = z
    return h, acts


def mixture(raw):
    raw = np.asarray(raw, np.float64).reshape(-1, LOBES, 5)
    m = raw[..., 0:3]
    ln = np.maximum(np.linalg.norm(m, axis=-1, keepdims=True), 1e-6)
    mu = m / ln
    kappa = np.exp(np.clip(raw[..., 3], -4.0, 7.0))
    lg = raw[..., 4] - raw[..., 4].max(-1, keepdims=True)
    w = np.exp(lg)
    w /= w.sum(-1, keepdims=True)
    return mu, kappa, w


def vmf_pdf(wdir, mu, kappa):
    norm = kappa / (2.0 * np.pi * -np.expm1(-2.0 * kappa))
    return norm * np.exp(kappa * (np.einsum("...j,...j->...", mu, wdir) - 1.0))


def mixture_pdf(raw, wdir):
    mu, kappa, w = mixture(raw)
    return np.sum(w * vmf_pdf(np.asarray(wdir)[:, None, :], mu, kappa), -1)


def loss(p, x, wdir, c, emulate_bf16=False):
    raw, _ = forward(p, x, emulate_bf16)
    q = np.maximum(mixture_pdf(raw, wdir), 1e-30)
    c = np.asarray(c, np.float64)
    return float(np.sum(c * -np.log(q)) / np.sum(c))


def grad(p, x, wdir, c, emulate_bf16=True):
    """Analytic gradient of loss() by backpropagation (hidden activations as stored)."""
    L = unpack(p)
    q = bf16 if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    raw, acts = forward(p, x, emulate_bf16)
    c = np.asarray(c, np.float64) / np.sum(c)
    r = raw.reshape(-1, LOBES, 5)
    m = r[..., 0:3]
    ln = np.maximum(np.linalg.norm(m, axis=-1, keepdims=True), 1e-6)
    mu = m / ln
    kr = r[..., 3]
    kap = np.exp(np.clip(kr, -4.0, 7.0))
    lg = r[..., 4] - r[..., 4].max(-1, keepdims=True)
    wk = np.exp(lg)
    wk /= wk.sum(-1, keepdims=True)
    wd = np.asarray(wdir, np.float64)[:, None, :]
    v = vmf_pdf(wd, mu, kap)
    pm = np.maximum(np.sum(wk * v, -1, keepdims=True), 1e-30)
    a = -c[:, None] / pm
    dv = a * wk
    dlogv = 1.0 / kap - 2.0 / np.expm1(2.0 * kap) + (np.sum(mu * wd, -1) - 1.0)
    g = np.zeros_like(r)
    g[..., 3] = np.where((kr > -4.0) & (kr < 7.0), dv * v * dlogv * kap, 0.0)
    gmu = wd * (dv * v * kap)[..., None]
    g[..., 0:3] = (gmu - mu * np.sum(mu * gmu, -1, keepdims=True)) / ln
    g[..., 4] = a * wk * (v - pm)
    dy = g.reshape(-1, OUT)
    grads = []
    for li in range(3, -1, -1):
        W, b = L[li]
        h_in = acts[li]
        # the device feeds dY to the tensor core as bf16 (weight gradient and dX); the
        # bias gradient sums the fp32 dY
        grads.append((q(dy).T @ h_in, dy.sum(0)))
        if li > 0:
            dx = q(dy) @ q(W)
            dy = dx * (acts[li] > 0)
    grads = grads[::-1]
    out = []
    for gW, gb in grads:
        out += [gW.reshape(-1), gb]
    return np.concatenate(out)


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for o, i in SHAPES:
        s = np.sqrt(6.0 / i)
        W = rng.uniform(-s, s, (o, i))
        if o == OUT:
            W *= 0.1
        out += [W.reshape(-1), np.zeros(o)]
    return np.concatenate(out).astype(np.float32)
