"""The renderer's random numbers: Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC 2011),
the counter-based generator that replaces the reference's per-thread MT19937 streams
(core/random.cc:70-163 behind Sampler::get1D / get2D, core/sampler.h:24-37).

CPU: the numpy restatement (oracle/philox.py) against the known-answer vectors that
the authors publish with their Random123 library, and the Sampler mirror's dimension
map.  GPU: the device generator (spgpu_sampler_generate) against the same vectors and
the restatement, and the Sampler mirror's get1D / get2D against the renderer's draws.
"""
import numpy as np
import pytest

from oracle import philox as P

# Random123's published known answers for philox4x32 with 10 rounds: counter, key -> output
KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def _kat_arrays():
    c = np.array([k[0] for k in KAT], np.uint32)
    k = np.array([k[1] for k in KAT], np.uint32)
    out = np.array([k_[2] for k_ in KAT], np.uint32)
    return c, k, out


def test_restatement_known_answers():
    c, k, out = _kat_arrays()
    assert np.array_equal(P.philox4x32_10(c, k), out)


def test_uniforms_in_unit_interval():
    w = np.array([0, 255, 256, 0xFFFFFFFF], np.uint32)
    u = P.u01(w)
    assert u[0] == 0.0 and u[1] == 0.0 and u[2] == 2.0 ** -24 and u[3] == 1.0 - 2.0 ** -24
    assert u.dtype == np.float32


def test_sampler_dimension_map():
    from spica_gb300.gpu import CAMERA_BOUNCE, GpuSampler
    assert [GpuSampler.block_of(d) for d in range(4)] == [(CAMERA_BOUNCE, 0, d) for d in range(4)]
    assert GpuSampler.block_of(4) == (0, 0, 0)
    assert GpuSampler.block_of(4 + 5) == (0, 1, 1)
    assert GpuSampler.block_of(4 + 16 * 3 + 4 * 2 + 3) == (3, 2, 3)


@pytest.mark.gpu
def test_device_known_answers_and_restatement(gpulib):
    from spica_gb300 import philox
    c, k, out = _kat_arrays()
    raw, u = philox(c, k)
    assert np.array_equal(raw, out)
    assert np.array_equal(u, P.u01(out))
    rng = np.random.default_rng(11)
    n = 1 << 18
    c = rng.integers(0, 1 << 32, size=(n, 4), dtype=np.uint64).astype(np.uint32)
    k = rng.integers(0, 1 << 32, size=(n, 2), dtype=np.uint64).astype(np.uint32)
    raw, u = philox(c, k)
    assert np.array_equal(raw, P.philox4x32_10(c, k))
    assert np.array_equal(u, P.u01(raw))


@pytest.mark.gpu
def test_renderer_streams_are_uniform(gpulib):
    """The renderer's draws over a film of keys and a run of samples: mean 1/2, variance
    1/12, a flat 64-bin histogram (chi-square), and no correlation between neighbouring
    lanes or pixels."""
    from spica_gb300 import philox
    npix, ns = 4096, 64
    pix, smp = np.meshgrid(np.arange(npix, dtype=np.uint32), np.arange(ns, dtype=np.uint32), indexing="ij")
    ctr = np.stack([smp.ravel(), np.zeros(npix * ns, np.uint32), np.full(npix * ns, 1, np.uint32),
                    np.full(npix * ns, P.STREAM_TAG, np.uint32)], 1)
    key = np.stack([np.full(npix * ns, 7, np.uint32), pix.ravel()], 1)
    _, u = philox(ctr, key)
    x = u.astype(np.float64).ravel()
    n = x.size
    assert abs(x.mean() - 0.5) < 5 * np.sqrt(1 / 12 / n)
    assert abs(x.var() - 1 / 12) < 5 * np.sqrt(1 / 180 / n)
    h, _ = np.histogram(x, bins=64, range=(0, 1))
    chi2 = ((h - n / 64) ** 2 / (n / 64)).sum()
    assert chi2 < 63 + 5 * np.sqrt(2 * 63)
    for a, b in ((u[:, 0], u[:, 1]), (u[:, 2], u[:, 3]), (u[:-1, 0], u[1:, 0])):
        r = np.corrcoef(a, b)[0, 1]
        assert abs(r) < 5 / np.sqrt(a.size)


@pytest.mark.gpu
def test_sampler_mirror_matches_renderer_draws(gpulib):
    """GpuSampler (startPixel / startNextSample / get1D / get2D / clone) returns, dimension
    by dimension, the numbers the renderer draws for that pixel and sample."""
    from spica_gb300 import GpuSampler
    s = GpuSampler(seed=1234, width=64)
    s.startPixel(5, 3)
    px = 3 * 64 + 5
    for sample in range(3):
        s.startNextSample()
        got = [s.get1D() for _ in range(4)] + list(s.get2D()) + [s.get1D() for _ in range(70)]
        want = [P.renderer_draws(1234, px, sample, P.CAMERA_BOUNCE, 0)[d] for d in range(4)]
        for d in range(4, 4 + 72):
            b, st, lane = GpuSampler.block_of(d)
            want.append(P.renderer_draws(1234, px, sample, b, st)[lane])
        assert np.array_equal(np.array(got, np.float32), np.array(want, np.float32))
    c = s.clone(99)
    c.startPixel(px)
    c.startNextSample()
    assert c.get1D() == float(P.renderer_draws(99, px, 0, P.CAMERA_BOUNCE, 0)[0])
