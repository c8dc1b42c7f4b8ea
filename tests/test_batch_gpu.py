"""Batched uneven renders in one persistent launch: every film of the batch equals the
same scene rendered alone by the wavefront integrator (same random streams, same
estimator; only the order of floating-point additions differs), and the per-render
completion times are reported."""
import numpy as np
import pytest

from spica_gb300 import GpuBatch, GpuBVHAccel, GpuPathIntegrator, scenes

pytestmark = pytest.mark.gpu


def small_variants(n=6, seed=4):
    vs = scenes.batch_variants(n, seed=seed)
    for k, v in enumerate(vs):   # keep the test fast: small films, few samples
        v.width = v.height = 32 + 32 * (k % 3)
        v.spp = 8 + 4 * (k % 4)
    return vs


@pytest.mark.parametrize("autotune", [False, True])
def test_batch_matches_individual_renders(gpulib, autotune):
    import torch
    vs = small_variants()
    b = GpuBatch(vs, seed=21, autotune=autotune)
    films = torch.zeros((b.pixels, 4), dtype=torch.float32, device="cuda")
    ms, st = b.run(films)
    torch.cuda.synchronize()
    host = films.cpu().numpy()
    assert st.paths == sum(v.width * v.height * v.spp for v in vs)
    assert np.all(ms > 0) and np.all(ms <= st.ms * 1.01 + 1.0)
    if autotune:
        assert b.tuning.candidates > 1 and b.tuning.block in (64, 128, 256)
    for i, v in enumerate(vs):
        acc = GpuBVHAccel(v).construct()
        ref = GpuPathIntegrator(seed=21).render(v.camera, acc, {"width": v.width, "height": v.height,
                                                                "maxDepth": v.max_depth, "sampleCount": v.spp})
        got = b.film(host, i)
        assert np.array_equal(got[..., 3], ref[..., 3])
        np.testing.assert_allclose(got[..., :3], ref[..., :3], rtol=2e-4, atol=2e-4)


def test_batch_rerun_accumulates(gpulib):
    import torch
    vs = small_variants(3, seed=9)
    b = GpuBatch(vs, seed=2, autotune=False)
    films = torch.zeros((b.pixels, 4), dtype=torch.float32, device="cuda")
    b.run(films)
    b.run(films)
    torch.cuda.synchronize()
    host = films.cpu().numpy()
    for i, v in enumerate(vs):
        assert np.all(b.film(host, i)[..., 3] == 2 * v.spp)
