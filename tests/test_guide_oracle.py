"""The CPU oracle of the guiding network: analytic gradient against finite differences,
mixture density normalisation, BF16 rounding."""
import numpy as np

from oracle import guide_oracle as go


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = go.init_params(1).astype(np.float64)
    p[go.N_PARAMS - 40:] = rng.normal(size=40) * 0.3
    n = 48
    x = rng.random((n, 9))
    w = rng.normal(size=(n, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    c = rng.random(n) + 0.1
    g = go.grad(p, x, w, c, emulate_bf16=False)
    for i in rng.choice(go.N_PARAMS, 30, replace=False):
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        fd = (go.loss(pp, x, w, c) - go.loss(pm, x, w, c)) / (2 * e)
        assert abs(fd - g[i]) <= 1e-3 * abs(fd) + 1e-6, (i, fd, g[i])


def test_mixture_density_integrates_to_one():
    rng = np.random.default_rng(1)
    raw = rng.normal(size=(1, 40)) * 2.0
    z = rng.random(200000) * 2 - 1
    ph = rng.random(200000) * 2 * np.pi
    s = np.sqrt(1 - z * z)
    dirs = np.stack([s * np.cos(ph), s * np.sin(ph), z], 1)
    est = 4 * np.pi * np.mean(go.mixture_pdf(np.repeat(raw, dirs.shape[0], 0), dirs))
    assert abs(est - 1.0) < 0.03


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.0078125, -3.14159, 65504.0], np.float32)
    r = go.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-6
