"""Batched uneven renders in one graph launch, on either engine (the streaming
wavefront over all renders, the persistent megakernel): every film of the batch equals
the same scene rendered alone by the wavefront integrator (same random streams, same
estimator; only the order of floating-point additions differs), and the per-render
completion times are reported."""
import numpy as np
import pytest

from spica_gb300 import GpuBatch, GpuBVHAccel, GpuPathIntegrator, scenes
from spica_gb300.gpu import BATCH_PERSISTENT, BATCH_STREAM

pytestmark = pytest.mark.gpu


def small_variants(n=6, seed=4):
    vs = scenes.batch_variants(n, seed=seed)
    for k, v in enumerate(vs):   # keep the test fast: small films, few samples
        v.width = v.height = 32 + 32 * (k % 3)
        v.spp = 8 + 4 * (k % 4)
    return vs


@pytest.mark.parametrize("autotune", [0, 1, BATCH_PERSISTENT])
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
    assert st.kernel_launches > 0
    if autotune == 1:
        assert b.tuning.candidates > 1 and b.tuning.engine in (BATCH_STREAM, BATCH_PERSISTENT)
    else:
        assert b.tuning.engine == (BATCH_PERSISTENT if autotune == BATCH_PERSISTENT else BATCH_STREAM)
    if b.tuning.engine == BATCH_PERSISTENT:
        assert b.tuning.block in (64, 128, 256)
    else:
        assert b.tuning.pool_slots > 0 and b.tuning.pool_lanes in (1, 2) and b.tuning.iterations > 0
    for i, v in enumerate(vs):
        acc = GpuBVHAccel(v).construct()
        ref = GpuPathIntegrator(seed=21).render(v.camera, acc, {"width": v.width, "height": v.height,
                                                                "maxDepth": v.max_depth, "sampleCount": v.spp})
        got = b.film(host, i)
        assert np.array_equal(got[..., 3], ref[..., 3])
        np.testing.assert_allclose(got[..., :3], ref[..., :3], rtol=2e-4, atol=2e-4)


@pytest.mark.parametrize("autotune", [0, BATCH_PERSISTENT])
def test_batch_rerun_accumulates(gpulib, autotune):
    import torch
    vs = small_variants(3, seed=9)
    b = GpuBatch(vs, seed=2, autotune=autotune)
    films = torch.zeros((b.pixels, 4), dtype=torch.float32, device="cuda")
    b.run(films)
    b.run(films)
    torch.cuda.synchronize()
    host = films.cpu().numpy()
    for i, v in enumerate(vs):
        assert np.all(b.film(host, i)[..., 3] == 2 * v.spp)
    # a second film: the graph is rebuilt for the new address
    other = torch.zeros_like(films)
    b.run(other)
    torch.cuda.synchronize()
    for i, v in enumerate(vs):
        assert np.all(b.film(other.cpu().numpy(), i)[..., 3] == v.spp)


def test_streaming_batch_many_renders_small_pool(gpulib):
    """A streaming batch whose pool is smaller than any render: renders share the pool,
    paths of consecutive renders are in flight together, and every film is complete."""
    import torch
    vs = scenes.batch_variants(12, seed=31)
    for k, v in enumerate(vs):
        v.width = v.height = 32 + 16 * (k % 4)
        v.spp = 4 + 2 * (k % 3)
    b = GpuBatch(vs, seed=5, autotune=0, pool=(4096, 2))
    assert b.tuning.engine == BATCH_STREAM and b.tuning.pool_slots == 4096 and b.tuning.pool_lanes == 2
    films = torch.zeros((b.pixels, 4), dtype=torch.float32, device="cuda")
    ms, st = b.run(films)
    torch.cuda.synchronize()
    host = films.cpu().numpy()
    assert st.paths == sum(v.width * v.height * v.spp for v in vs)
    assert np.all(ms > 0)
    for i, v in enumerate(vs):
        got = b.film(host, i)
        assert np.all(got[..., 3] == v.spp)
        acc = GpuBVHAccel(v).construct()
        ref = GpuPathIntegrator(seed=5).render(v.camera, acc, {"width": v.width, "height": v.height,
                                                               "maxDepth": v.max_depth, "sampleCount": v.spp})
        np.testing.assert_allclose(got[..., :3], ref[..., :3], rtol=2e-4, atol=2e-4)


def test_batch_profile_matches_run(gpulib):
    """The host-driven profile of a streaming batch traces the same paths as its graph
    run (same counts, same films up to summation order) and times every kernel class;
    a persistent batch has no such profile."""
    import torch
    from spica_gb300 import SpgpuError
    from spica_gb300.gpu import KERNEL_CLASSES
    vs = small_variants(4, seed=13)
    b = GpuBatch(vs, seed=3, autotune=0, pool=(8192, 2))
    films = torch.zeros((b.pixels, 4), dtype=torch.float32, device="cuda")
    _, st = b.run(films)
    prof_films = torch.zeros_like(films)
    pr = b.profile(prof_films)
    torch.cuda.synchronize()
    assert pr.paths == st.paths and pr.rays_closest == st.rays_closest and pr.rays_shadow == st.rays_shadow
    assert all(pr.launches[k] > 0 and pr.kernel_ms[k] > 0 for k in range(len(KERNEL_CLASSES)))
    assert pr.closest_nodes_per_ray > 0
    a, p2 = films.cpu().numpy(), prof_films.cpu().numpy() / 2   # the profile renders twice
    np.testing.assert_array_equal(a[:, 3], p2[:, 3])
    np.testing.assert_allclose(a[:, :3], p2[:, :3], rtol=2e-4, atol=2e-4)
    bp = GpuBatch(vs, seed=3, autotune=BATCH_PERSISTENT)
    with pytest.raises(SpgpuError):
        bp.profile(films)


@pytest.mark.parametrize("autotune", [0, BATCH_PERSISTENT])
def test_batch_edge_shapes(gpulib, autotune):
    """A batch of one render, and a batch whose renders differ in maximum depth (0, 1, 3
    and 8) and take 1 to 3 samples per pixel: each film equals the same scene rendered
    alone."""
    import torch
    for vs in ([small_variants(1, seed=2)[0]], small_variants(4, seed=6)):
        for k, v in enumerate(vs):
            v.max_depth = [8, 0, 1, 3][k % 4]
            v.spp = 1 + k % 3
        b = GpuBatch(vs, seed=17, autotune=autotune)
        films = torch.zeros((b.pixels, 4), dtype=torch.float32, device="cuda")
        ms, st = b.run(films)
        torch.cuda.synchronize()
        host = films.cpu().numpy()
        assert st.paths == sum(v.width * v.height * v.spp for v in vs)
        assert np.all(ms > 0)
        for i, v in enumerate(vs):
            acc = GpuBVHAccel(v).construct()
            ref = GpuPathIntegrator(seed=17).render(v.camera, acc, {"width": v.width, "height": v.height,
                                                                    "maxDepth": v.max_depth, "sampleCount": v.spp})
            got = b.film(host, i)
            assert np.array_equal(got[..., 3], ref[..., 3])
            np.testing.assert_allclose(got[..., :3], ref[..., :3], rtol=2e-4, atol=2e-4)
