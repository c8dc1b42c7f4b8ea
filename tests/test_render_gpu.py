"""Rendered images of the GPU wavefront path integrator against the reference
renderer (golden per-pixel sums from the compiled reference) and the CPU oracle:
per-pixel mean within 3 sigma (tests/parity.py), and relMSE decaying as 1/spp."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from parity import zscores
from spica_gb300 import GpuBVHAccel, GpuPathIntegrator, scenes
from spica_gb300.gpu import GpuDirectLightingIntegrator

pytestmark = pytest.mark.gpu


class _S:
    pass


def _scene_from(g):
    s = _S()
    for k in ("verts", "tri_mat", "materials", "tri_emit", "env"):
        setattr(s, k, g[k])
    return s


def gpu_batches(accel, camera, W, H, max_depth, batches, spp, seed=1, integrator=GpuPathIntegrator):
    """Independent batch means -> per-pixel mean and variance of the mean."""
    integ = integrator(seed=seed)
    means = []
    for k in range(batches):
        film = integ.render(camera, accel, {"width": W, "height": H, "maxDepth": max_depth, "sampleCount": spp},
                            sample_offset=k * spp)
        assert np.all(film[..., 3] == spp)
        means.append(film[..., :3] / spp)
    m = np.stack(means)
    return m.mean(0), m.var(0, ddof=1) / batches


def ref_moments(g):
    """Per-pixel mean and variance of the mean of a reference render: from independent
    batch means where the fixture holds them, else from the per-sample sums."""
    if "bmean" in g:
        return g["bmean"], g["bvar"]
    n = float(g["spp"])
    mean = g["sum"] / n
    var = np.maximum(g["sumsq"] / n - mean ** 2, 0.0) * n / (n - 1) / n
    return mean, var


@pytest.mark.parametrize("name", ["render_boxroom", "render_envscene", "render_direct_boxroom",
                                  "render_direct_envscene", "render_material_room",
                                  "render_direct_material_room", "render_conductor_room"])
def test_matches_reference_render(gpulib, name):
    """Path integrator and direct-lighting integrator against the reference's renders."""
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    W, H, md = int(g["W"]), int(g["H"]), int(g["max_depth"])
    if "material_room" in name:   # rough dielectric and plastic boxes
        sc = scenes.material_room(width=W, height=H)
    elif "conductor_room" in name:   # Beckmann and GGX rough conductor boxes
        sc = scenes.conductor_room(width=W, height=H)
    else:
        sc = scenes.box_room(width=W, height=H) if "boxroom" in name else _scene_from(g)
    acc = GpuBVHAccel(sc).construct()
    integ = GpuDirectLightingIntegrator if "direct" in name else GpuPathIntegrator
    # match the fixture's sample count where it holds batch moments: both sides then see
    # the same share of the rare bright paths through the glass box
    batches, spp = (int(g["batches"]), int(g["batch_spp"])) if "bmean" in g else (16, 512)
    mg, vg = gpu_batches(acc, g["camera"], W, H, md, batches=batches, spp=spp, integrator=integ)
    mr, vr = ref_moments(g)
    z = zscores(mg, vg, mr, vr)
    frac = float((np.abs(z) > 3).mean())
    dump = os.environ.get("SPICA_TEST_DUMP")
    if dump:
        np.savez_compressed(os.path.join(dump, f"{name}_gpu.npz"), mg=mg, vg=vg, mr=mr, vr=vr, z=z)
    worst = np.unravel_index(np.argmax(np.abs(z)), z.shape)
    assert frac < 0.01, (frac, float(np.abs(z).max()), float(z.mean()), worst, float(mg[worst]), float(mr[worst]))
    # image mean within 3 standard errors
    se = np.sqrt(vg.sum() + vr.sum()) / z.size
    assert abs(mg.mean() - mr.mean()) < 3 * se + 1e-6, (mg.mean(), mr.mean(), se)


def test_relmse_decays_as_one_over_spp(gpulib):
    sc = scenes.box_room(width=64, height=64)
    acc = GpuBVHAccel(sc).construct()
    integ = GpuPathIntegrator(seed=99)
    p = {"width": 64, "height": 64, "maxDepth": 8}
    ref = integ.render(sc.camera, acc, dict(p, sampleCount=16384), sample_offset=1 << 20)
    R = ref[..., :3] / ref[..., 3:]
    spps = [16, 64, 256, 1024]
    rel = []
    for i, s in enumerate(spps):
        errs = []
        for rep in range(4):
            f = GpuPathIntegrator(seed=1000 + rep).render(sc.camera, acc, dict(p, sampleCount=s))
            I = f[..., :3] / f[..., 3:]
            errs.append(np.mean((I - R) ** 2 / (R ** 2 + 1e-2)))
        rel.append(np.mean(errs))
    slope = np.polyfit(np.log(spps), np.log(rel), 1)[0]
    assert -1.1 <= slope <= -0.9, (slope, rel)


def test_render_edge_cases(gpulib):
    sc = scenes.box_room(width=8, height=8)
    acc = GpuBVHAccel(sc).construct()
    integ = GpuPathIntegrator(seed=3)
    f0 = integ.render(sc.camera, acc, {"width": 8, "height": 8, "maxDepth": 8, "sampleCount": 0})
    assert not f0.any()
    # maxDepth 0: only emission seen directly
    f = integ.render(sc.camera, acc, {"width": 33, "height": 17, "maxDepth": 0, "sampleCount": 8})
    assert np.all(f[..., 3] == 8)
    lum = f[..., :3].sum(-1)
    assert lum.max() > 0 and (lum == 0).mean() > 0.5
    # 1 x 1 film, accumulation across calls
    a = integ.render(sc.camera, acc, {"width": 1, "height": 1, "maxDepth": 8, "sampleCount": 4})
    integ.render(sc.camera, acc, {"width": 1, "height": 1, "maxDepth": 8, "sampleCount": 4}, film=a, sample_offset=4)
    assert a[0, 0, 3] == 8


def test_pass_lanes_render_the_same_samples(gpulib):
    """Concurrent sample passes (pass lanes, each with its own queues and stream) render
    exactly the samples a single lane renders: per-pixel sums agree up to the order of
    the film's atomic additions, for spp below, at and above the lane count."""
    from spica_gb300.gpu import Context
    sc = scenes.box_room(width=96, height=64)
    params = {"width": 96, "height": 64, "maxDepth": 8}
    integ = GpuPathIntegrator(seed=21)
    films = {}
    for lanes in (1, 3, 8):
        acc = GpuBVHAccel(sc, ctx=Context(0, pass_lanes=lanes, wavefront=1)).construct()
        films[lanes] = [integ.render(sc.camera, acc, dict(params, sampleCount=spp), sample_offset=5)
                        for spp in (2, 3, 11)]
    for lanes in (3, 8):
        for a, b in zip(films[1], films[lanes]):
            np.testing.assert_array_equal(a[..., 3], b[..., 3])
            np.testing.assert_allclose(a[..., :3], b[..., :3], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("scene", ["box_room", "material_room", "mid_scale"])
def test_streaming_and_pass_by_pass_render_the_same_samples(gpulib, scene):
    """The streaming wavefront (path pool refilled as paths end, the default) and the
    pass-by-pass wavefront draw the same numbers for every (pixel, sample, depth), so
    their films agree up to the order of the film's atomic additions: on the box room,
    on the material room (rough dielectric, plastic) and on a 320 x 180 crop of the
    mid-scale scene (environment map, conductors, glass), for spp below and above what
    fills the pool, and for the direct-lighting integrator."""
    from spica_gb300.gpu import Context
    if scene == "mid_scale":
        sc = scenes.mid_scale(width=320, height=180)
    else:
        sc = getattr(scenes, scene)(width=96, height=64)
    params = {"width": sc.width, "height": sc.height, "maxDepth": sc.max_depth}
    films = {}
    for wf in (0, 1):
        acc = GpuBVHAccel(sc, ctx=Context(0, wavefront=wf)).construct()
        out = []
        for integ, spp in ((GpuPathIntegrator(seed=8), 3), (GpuPathIntegrator(seed=9), 40),
                           (GpuDirectLightingIntegrator(seed=10), 5)):
            out.append(integ.render(sc.camera, acc, dict(params, sampleCount=spp), sample_offset=7))
            st = integ.last_stats
            assert st.paths == spp * sc.width * sc.height
            out.append(np.array([st.paths, st.rays_closest, st.rays_shadow], np.float64))
        films[wf] = out
    for a, b in zip(films[0], films[1]):
        if a.ndim == 1:   # path and ray counts: the same paths, the same rays
            np.testing.assert_array_equal(a, b)
            continue
        np.testing.assert_array_equal(a[..., 3], b[..., 3])
        scale = float(np.abs(b[..., :3]).max())
        close = np.abs(a[..., :3] - b[..., :3]) <= 1e-5 * np.abs(b[..., :3]) + 1e-6 * scale
        assert close.mean() > 0.999, close.mean()


def test_streaming_pool_refills_within_a_sample(gpulib):
    """A film larger than a streaming pool (4096 x 2304 = 9.4M pixels, 2^23 path slots per
    pool): each pool refills while its sample is still in flight, and the film holds the
    same samples as the pass-by-pass wavefront's: every pixel's count, the path and ray
    counts, and the sums up to the order of the film's additions."""
    from spica_gb300.gpu import Context
    sc = scenes.box_room(width=4096, height=2304)
    params = {"width": 4096, "height": 2304, "maxDepth": 8, "sampleCount": 2}
    out = {}
    for wf in (0, 1):
        acc = GpuBVHAccel(sc, ctx=Context(0, pass_lanes=1, wavefront=wf)).construct()
        integ = GpuPathIntegrator(seed=17)
        film = integ.render(sc.camera, acc, params, sample_offset=3)
        st = integ.last_stats
        out[wf] = (film, (st.paths, st.rays_closest, st.rays_shadow), st.kernel_launches)
    (fs, ss, ls), (fp, sp, lp) = out[0], out[1]
    assert ss == sp and ss[0] == 2 * 4096 * 2304
    # streaming: replays of 8 iterations of 7 kernels; pass by pass: 2 + 5 (depth + 1) per pass
    assert ls > 0 and ls % 56 == 0 and lp == 2 * (2 + 5 * 9)
    np.testing.assert_array_equal(fs[..., 3], fp[..., 3])
    assert np.all(fs[..., 3] == 2)
    scale = float(np.abs(fp[..., :3]).max())
    close = np.abs(fs[..., :3] - fp[..., :3]) <= 1e-5 * np.abs(fp[..., :3]) + 1e-6 * scale
    assert close.mean() > 0.999, close.mean()


def test_checkpoint_resume_continues_the_sample_index(gpulib, tmp_path):
    """Checkpoint / resume: the film (sum of L, sample count) saved after k samples and
    rendered on from sample_offset = k holds exactly the samples of one uninterrupted
    render (the sampler is counter-based: a sample's numbers depend only on its
    pixel, index, bounce and stream)."""
    sc = scenes.box_room(width=80, height=60)
    params = {"width": 80, "height": 60, "maxDepth": 8}
    acc = GpuBVHAccel(sc).construct()
    integ = GpuPathIntegrator(seed=5)
    whole = integ.render(sc.camera, acc, dict(params, sampleCount=12))
    part = integ.render(sc.camera, acc, dict(params, sampleCount=5))
    np.save(tmp_path / "film.npy", part)                       # checkpoint
    film = np.load(tmp_path / "film.npy")                      # resume
    integ.render(sc.camera, acc, dict(params, sampleCount=7), film=film, sample_offset=5)
    np.testing.assert_array_equal(film[..., 3], whole[..., 3])
    np.testing.assert_allclose(film[..., :3], whole[..., :3], rtol=1e-5, atol=1e-6)
