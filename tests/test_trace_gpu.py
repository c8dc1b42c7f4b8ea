"""Closest-hit and any-hit traversal of the device-built wide BVH against the
reference (golden fixtures from the compiled reference) and the CPU oracle, through
the C ABI.  Rules in tests/parity.py."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from parity import classify_any, classify_closest
from spica_gb300 import GpuBVHAccel, scenes

pytestmark = pytest.mark.gpu


class _S:
    pass


def _tri_scene(v):
    s = _S()
    s.verts = np.asarray(v, np.float32).reshape(-1, 9)
    s.tri_mat = np.zeros(s.verts.shape[0], np.int32)
    s.materials = np.array([scenes.lambert(0.5, 0.5, 0.5)])
    s.tri_emit = s.env = None
    return s


def test_triangle_kat_gpu(gpulib):
    kat = json.load(open(os.path.join(GOLDEN, "kat_triangle.json")))
    acc = GpuBVHAccel(_tri_scene(kat["triangle"])).construct()
    d = np.array(kat["hit_ray"]["dir_unnormalised"], np.float64)
    d /= np.linalg.norm(d)
    prim, t, u, v = acc.intersect(np.array([kat["hit_ray"]["org"]]), d[None])
    assert prim[0] == 0
    assert abs(t[0] - math.sqrt(6.0) / 2.0) <= 1e-6 * math.sqrt(6.0) / 2.0
    mp, *_ = acc.intersect(np.array(kat["miss_rays"]["orgs"]), np.tile(kat["miss_rays"]["dir"], (4, 1)))
    assert list(mp) == [-1, -1, -1, -1]
    assert not acc.intersect_any(np.array(kat["miss_rays"]["orgs"]), np.tile(kat["miss_rays"]["dir"], (4, 1))).any()
    assert acc.intersect_any(np.array([kat["hit_ray"]["org"]]), d[None]).all()


def test_golden_reference_trace(gpulib):
    """Primitive ids bit-exact vs the reference BVH except stated FP32 ties; t 1e-5."""
    g = np.load(os.path.join(GOLDEN, "trace_sphere.npz"))
    s = _S()
    s.verts, s.tri_mat = g["verts"], np.zeros(g["verts"].shape[0], np.int32)
    s.materials, s.tri_emit, s.env = np.array([scenes.lambert(0.5, 0.5, 0.5)]), None, None
    acc = GpuBVHAccel(s).construct()
    prim, t, _, _ = acc.intersect(g["org"], g["dir"])
    r = classify_closest(g["verts"], g["org"], g["dir"], prim, t, g["prim"], g["t"])
    assert r["fail"] == 0, r
    assert r["t_fail"] == 0, r
    assert r["equal"] >= 0.995 * r["total"], r
    h = acc.intersect_any(g["org"], g["dir"], g["tmax"])
    ra = classify_any(g["verts"], g["org"], g["dir"], g["tmax"], h, g["any"], g["prim"], g["t"], prim, t)
    assert ra["fail"] == 0, ra


@pytest.mark.parametrize("levels", [6, 9])
def test_microbench_scene_vs_oracle(gpulib, port, levels):
    """The intersection-microbench sphere (levels=9: 1,048,576 triangles) with a
    seeded subset of its coherent and incoherent rays, against the CPU oracle."""
    sph = scenes.displaced_sphere(levels=levels, seed=0)
    n_half = 40_000 if levels == 9 else 20_000
    org, d, tmax = scenes.microbench_rays(sph, n_half, n_half, 4096, 2048, seed=1)
    acc = GpuBVHAccel(sph).construct()
    info = acc.info()
    assert info.triangles == sph.ntri and info.depth >= 2
    prim, t, _, _ = acc.intersect(org, d)
    o = port.scene(sph)
    pr, tr = o.trace(org.astype(np.float64), d.astype(np.float64))
    r = classify_closest(sph.verts, org, d, prim, t, pr, tr)
    assert r["fail"] == 0 and r["t_fail"] == 0, r
    assert r["equal"] >= 0.995 * r["total"], r
    h = acc.intersect_any(org, d, tmax)
    hr = o.trace(org.astype(np.float64), d.astype(np.float64), tmax.astype(np.float64), any_hit=True)
    ra = classify_any(sph.verts, org, d, tmax, h, hr, pr, tr, prim, t)
    assert ra["fail"] == 0, ra


def test_device_entry_point_matches_host(gpulib):
    import torch
    sph = scenes.displaced_sphere(levels=5, seed=3)
    org, d, tmax = scenes.microbench_rays(sph, 5000, 5000, 128, 64, seed=2)
    acc = GpuBVHAccel(sph).construct()
    prim, t, u, v = acc.intersect(org, d)
    ot = torch.zeros((org.shape[0], 4), dtype=torch.float32, device="cuda")
    dt = torch.zeros_like(ot)
    ot[:, :3] = torch.from_numpy(org).cuda()
    dt[:, :3] = torch.from_numpy(d).cuda()
    dt[:, 3] = 1e32
    out = torch.zeros_like(ot)
    acc.intersect_device(ot, dt, out)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    assert np.array_equal(o[:, 1].view(np.int32), prim)
    assert np.array_equal(o[:, 0], t)
    anyo = torch.zeros(org.shape[0], dtype=torch.int32, device="cuda")
    dt[:, 3] = torch.from_numpy(tmax).cuda()
    acc.intersect_device(ot, dt, anyo, any_hit=True)
    torch.cuda.synchronize()
    assert np.array_equal(anyo.cpu().numpy().astype(bool), acc.intersect_any(org, d, tmax))
    c = acc.intersect_stats(ot, dt, out)
    assert c.rays == org.shape[0] and c.nodes_per_ray > 1 and c.tris_per_ray > 0


def test_edge_cases(gpulib):
    sph = scenes.displaced_sphere(levels=3, seed=1)
    acc = GpuBVHAccel(sph).construct()
    # empty batch
    p, t, u, v = acc.intersect(np.zeros((0, 3)), np.zeros((0, 3)))
    assert p.size == 0
    # tmax = 0: nothing can be hit; origin inside the sphere: everything is hit
    o = np.zeros((64, 3), np.float32)
    rng = np.random.default_rng(0)
    d = rng.normal(size=(64, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    assert not acc.intersect_any(o, d, np.zeros(64)).any()
    assert acc.intersect_any(o, d).all()
    p, t, *_ = acc.intersect(o, d)
    assert (p >= 0).all() and (t > 0.9).all() and (t < 1.1).all()
    # rays pointing away from everything miss
    p, *_ = acc.intersect(np.tile([0, 0, 5.0], (8, 1)), np.tile([0, 0, 1.0], (8, 1)))
    assert (p == -1).all()
    # single-triangle scene and axis-parallel rays
    one = GpuBVHAccel(_tri_scene([0, 0, 0, 1, 0, 0, 0, 1, 0])).construct()
    p, t, *_ = one.intersect(np.array([[0.25, 0.25, 1.0], [2.0, 2.0, 1.0]]), np.array([[0, 0, -1.0], [0, 0, -1.0]]))
    assert list(p) == [0, -1] and abs(t[0] - 1.0) < 1e-6


def test_invalid_arguments_raise(gpulib):
    from spica_gb300 import SpgpuError, gpu
    ctx = gpu.Context()
    with pytest.raises(SpgpuError):
        ctx.build_bvh()          # no scene yet
    bad = _tri_scene([0, 0, 0, 1, 0, 0, 0, 1, 0])
    bad.tri_mat = np.array([5], np.int32)
    with pytest.raises(SpgpuError):
        ctx.upload_scene(bad)    # material index out of range


def test_host_trace_from_many_threads(gpulib):
    """spgpu_trace_host called on one context from eight host threads at once, as the
    reference calls Accelerator::intersect from every render thread
    (core/integrator.cc:77): batches of 1 to 4096 rays, closest and any hit, each
    result identical to the same call made alone."""
    import threading
    sph = scenes.displaced_sphere(levels=6, seed=2)
    org, d, tmax = scenes.microbench_rays(sph, 20000, 20000, 256, 128, seed=4)
    acc = GpuBVHAccel(sph).construct()
    rng = np.random.default_rng(8)
    jobs = []
    i = 0
    while i < org.shape[0]:
        n = int(rng.choice([1, 1, 1, 7, 64, 4096]))
        jobs.append((i, min(i + n, org.shape[0]), bool(rng.integers(0, 2))))
        i += n
    alone = {}
    for a, b, anyh in jobs:
        alone[a] = acc.intersect_any(org[a:b], d[a:b], tmax[a:b]) if anyh else acc.intersect(org[a:b], d[a:b])[:2]
    got, errors = {}, []

    def worker(my):
        try:
            for a, b, anyh in my:
                got[a] = (acc.intersect_any(org[a:b], d[a:b], tmax[a:b]) if anyh
                          else acc.intersect(org[a:b], d[a:b])[:2])
        except Exception as e:   # noqa: BLE001 -- reported below
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(jobs[k::8],)) for k in range(8)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    assert len(got) == len(jobs)
    for a, b, anyh in jobs:
        if anyh:
            assert np.array_equal(got[a], alone[a])
        else:
            assert np.array_equal(got[a][0], alone[a][0]) and np.array_equal(got[a][1], alone[a][1])
