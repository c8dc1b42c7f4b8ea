"""Philox4x32-10 in numpy: the CPU restatement the device generator is checked against.

TEST INFRASTRUCTURE ONLY -- imported by tests/, never by the product package.

Written from the published algorithm (Salmon, Moraes, Dror and Shaw, "Parallel random
numbers: as easy as 1, 2, 3", SC 2011): ten rounds of two 32 x 32 -> 64-bit multiplies
with the multipliers 0xD2511F53 and 0xCD9E8D57, and a Weyl key schedule with the
increments 0x9E3779B9 and 0xBB67AE85 added after every round.  tests/test_sampler.py
pins it to the known-answer vectors the authors publish with their library.
"""
from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)
STREAM_TAG = 0x5350
CAMERA_BOUNCE = 0xFFFF


def philox4x32_10(counter, key):
    """counter (n, 4), key (n, 2) uint32 -> (n, 4) uint32."""
    c = np.asarray(counter, np.uint32).reshape(-1, 4).astype(np.uint64)
    k = np.asarray(key, np.uint32).reshape(-1, 2).copy()
    c0, c1, c2, c3 = c[:, 0], c[:, 1], c[:, 2], c[:, 3]
    k0, k1 = k[:, 0].astype(np.uint64), k[:, 1].astype(np.uint64)
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + np.uint64(W0)) & MASK
        k1 = (k1 + np.uint64(W1)) & MASK
    return np.stack([c0, c1, c2, c3], axis=1).astype(np.uint32)


def u01(words):
    """The renderer's uniform in [0, 1): the top 24 bits of a word times 2^-24 (exact in
    float32)."""
    return ((np.asarray(words, np.uint32) >> np.uint32(8)).astype(np.float64) * 2.0 ** -24).astype(np.float32)


def renderer_draws(seed, pixel, sample, bounce, stream):
    """The four uniforms the renderer draws for (seed, film pixel, sample, bounce, stream):
    key (seed, pixel), counter (sample, bounce, stream, 0x5350)."""
    n = np.broadcast(pixel, sample, bounce, stream).shape
    ctr = np.stack(np.broadcast_arrays(np.asarray(sample, np.uint32), np.asarray(bounce, np.uint32),
                                       np.asarray(stream, np.uint32), np.full(n, STREAM_TAG, np.uint32)), -1)
    key = np.stack(np.broadcast_arrays(np.full(n, seed, np.uint32), np.asarray(pixel, np.uint32)), -1)
    return u01(philox4x32_10(ctr.reshape(-1, 4), key.reshape(-1, 2))).reshape(*n, 4)
