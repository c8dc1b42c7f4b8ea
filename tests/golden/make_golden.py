"""Generate the golden fixtures in tests/golden/ from the reference renderer itself.

Runs the reference's own hot-path code, compiled unmodified by oracle/Makefile into
oracle/_ref/libspica_ref.so, so it needs the reference tree on this host:

    python tests/golden/make_golden.py

Fixtures (all small, committed):
  kat_triangle.json    the reference's triangle known-answer test
                       (tests/test_geometry.cc:50-77) run through BVHAccel
  trace_sphere.npz     a 4,096-triangle displaced sphere, 8,192 microbench rays and
                       the reference BVH's closest-hit primitive / t and any-hit bits
  bsdf_tables.npz      BSDF::f / pdf / sample of Lambert, GGX conductor and smooth
                       dielectric on seeded (wo, wi, u) sets
  render_boxroom.npz   per-pixel sum and sum of squares of PathIntegrator::Li on the
                       box room, 48 x 48 film, 1024 samples per pixel
  render_envscene.npz  the same on a small scene with an environment map, area
                       lights, conductors and dielectrics (scene arrays included)
"""
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import spo  # noqa: E402
from spica_gb300 import scenes  # noqa: E402


class _S:
    pass


def tri_scene(v):
    s = _S()
    s.verts = np.asarray(v, np.float64).reshape(1, 9)
    s.tri_mat = np.zeros(1, np.int32)
    s.materials = np.array([scenes.lambert(0.5, 0.5, 0.5)])
    s.tri_emit = None
    s.env = None
    return s


def bsdf_materials():
    return np.array([scenes.lambert(0.3, 0.5, 0.7),
                     scenes.conductor_f0(0.2, [0.6, 0.7, 0.95]),
                     scenes.conductor_f0(0.05, [0.9, 0.9, 0.9]),
                     scenes.dielectric(1.5)], np.float64)


def env_scene():
    return scenes.mid_scale(n_instances=30, seed=3, sphere_k=4, box_k=2, env_size=(256, 128), width=40, height=24,
                            spp=512, max_depth=16)


def main():
    spo.build("ref")
    ref = spo.Oracle("ref")
    t0 = time.time()

    # 1. triangle KAT of the reference's own test (tests/test_geometry.cc:50-77)
    s = ref.scene(tri_scene([1, 0, 0, 0, 0, 0, 0, 1, 0]))
    d = np.array([1.0, 1.0, 1.0]) - np.array([0.0, 0.0, -1.0])
    d /= np.linalg.norm(d)
    prim, t = s.trace(np.array([[0.0, 0.0, -1.0]]), d[None], nthreads=1)
    misses = [[-0.1, -0.1, 1.0], [0.6, 0.6, 1.0], [-0.1, 1.1, 1.0], [1.1, -0.1, 1.0]]
    mp, _ = s.trace(np.array(misses), np.tile([0.0, 0.0, -1.0], (4, 1)), nthreads=1)
    kat = {"source": "tests/test_geometry.cc:50-77 of the reference",
           "triangle": [1, 0, 0, 0, 0, 0, 0, 1, 0],
           "hit_ray": {"org": [0.0, 0.0, -1.0], "dir_unnormalised": [1.0, 1.0, 2.0],
                       "expected_t": math.sqrt(6.0) / 2.0, "reference_t": float(t[0]), "reference_prim": int(prim[0])},
           "miss_rays": {"orgs": misses, "dir": [0.0, 0.0, -1.0], "reference_prim": [int(x) for x in mp]}}
    with open(os.path.join(HERE, "kat_triangle.json"), "w") as f:
        json.dump(kat, f, indent=1)

    # 2. traversal on a small displaced sphere
    sph = scenes.displaced_sphere(levels=5, seed=0)
    org, dr, tmax = scenes.microbench_rays(sph, 4096, 4096, 128, 64, seed=5)
    s = ref.scene(sph)
    p, tt = s.trace(org.astype(np.float64), dr.astype(np.float64))
    h = s.trace(org.astype(np.float64), dr.astype(np.float64), tmax.astype(np.float64), any_hit=True)
    np.savez_compressed(os.path.join(HERE, "trace_sphere.npz"), verts=sph.verts, org=org, dir=dr, tmax=tmax,
                        prim=p, t=tt, any=h)

    # 3. BSDF tables
    rng = np.random.default_rng(11)
    n = 512
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    wi = rng.normal(size=(n, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    wi[: n // 2, 2] = np.abs(wi[: n // 2, 2]) * np.sign(wo[: n // 2, 2])   # half on wo's side
    u = rng.random((n, 2))
    mats = bsdf_materials()
    out = {"mats": mats, "wo": wo, "wi": wi, "u": u}
    for k, m in enumerate(mats):
        f, pdf = ref.bsdf_eval(m, wo, wi)
        swi, sf, spdf, st = ref.bsdf_sample(m, wo, u)
        out.update({f"f{k}": f, f"pdf{k}": pdf, f"swi{k}": swi, f"sf{k}": sf, f"spdf{k}": spdf, f"stype{k}": st})
    np.savez_compressed(os.path.join(HERE, "bsdf_tables.npz"), **out)

    # 4. box-room render
    sc = scenes.box_room(width=48, height=48, spp=1024)
    s = ref.scene(sc)
    S, S2 = s.render(sc.camera, 48, 48, 1024, 8, seed=7)
    np.savez_compressed(os.path.join(HERE, "render_boxroom.npz"), sum=S, sumsq=S2, spp=1024, seed=7, W=48, H=48,
                        max_depth=8, camera=sc.camera)

    # 5. environment-lit scene with conductors and dielectrics
    es = env_scene()
    s = ref.scene(es)
    S, S2 = s.render(es.camera, es.width, es.height, es.spp, es.max_depth, seed=13)
    np.savez_compressed(os.path.join(HERE, "render_envscene.npz"), sum=S, sumsq=S2, spp=es.spp, seed=13,
                        W=es.width, H=es.height, max_depth=es.max_depth, camera=es.camera, verts=es.verts,
                        tri_mat=es.tri_mat, materials=es.materials, tri_emit=es.tri_emit, env=es.env)
    direct_renders(ref)
    film_outputs(ref)
    more_materials(ref)
    conductors(ref)
    print(f"golden fixtures written in {time.time() - t0:.1f} s")


def direct_renders(ref):
    """6. the direct-lighting integrator on the same two scenes"""
    sc = scenes.box_room(width=48, height=48, spp=1024)
    S, S2 = ref.scene(sc).render(sc.camera, 48, 48, 1024, 8, seed=17, integrator="direct")
    np.savez_compressed(os.path.join(HERE, "render_direct_boxroom.npz"), sum=S, sumsq=S2, spp=1024, seed=17, W=48,
                        H=48, max_depth=8, camera=sc.camera)
    es = env_scene()
    S, S2 = ref.scene(es).render(es.camera, es.width, es.height, es.spp, es.max_depth, seed=19, integrator="direct")
    np.savez_compressed(os.path.join(HERE, "render_direct_envscene.npz"), sum=S, sumsq=S2, spp=es.spp, seed=19,
                        W=es.width, H=es.height, max_depth=es.max_depth, camera=es.camera, verts=es.verts,
                        tri_mat=es.tri_mat, materials=es.materials, tri_emit=es.tri_emit, env=es.env)


def film_input(W=131, H=37, seed=11):
    """A float film (sum of L, sample weight) covering the encoders' cases: zero and
    tiny pixels, values up to 1e6, unit and fractional weights, 131 columns so that an
    RGBE scanline needs two literal runs."""
    rng = np.random.default_rng(seed)
    w = rng.integers(1, 300, (H, W)).astype(np.float32)
    L = (10.0 ** rng.uniform(-6, 3, (H, W, 3))) * w[..., None]
    L[rng.random((H, W)) < 0.05] = 0.0
    L[0, :5] = [[1e-35, 1e-35, 1e-35], [1e6, 1e6, 1e6], [0, 0, 1], [1, 0, 0], [0.5, 0.25, 0.125]]
    w[0, :5] = 1.0
    return np.concatenate([L, w[..., None]], -1).astype(np.float32)


def film_outputs(ref):
    """7. film output: the reference's .hdr bytes, gamma 2.2 bytes and Reinhard image"""
    import tempfile
    film = film_input()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "film.hdr")
        ref.film_save_hdr(film, path)
        hdr = np.frombuffer(open(path, "rb").read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "film_output.npz"), film=film, hdr=hdr,
                        gamma22=ref.film_gamma(film, 2.2), reinhard=ref.film_reinhard(film, 0.18),
                        drago=ref.film_drago(film, 0.85), durand=ref.film_durand(film, 5.0))


def more_materials(ref):
    """8. rough dielectric (Beckmann, GGX) and plastic: BSDF tables, and path / direct renders
    of the material room.  One thread (a fresh one), so that the reference's hidden BxDF
    generators start from their seed and the fixtures are reproducible."""
    rng = np.random.default_rng(21)
    n = 2000
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    wi = rng.normal(size=(n, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    u = rng.random((n, 2))
    mats = np.array([scenes.rough_dielectric(0.3, 1.5, "beckmann"), scenes.rough_dielectric(0.15, 1.33, "ggx"),
                     scenes.plastic((0.6, 0.3, 0.2), (0.4, 0.4, 0.4), 1.5),
                     scenes.plastic((0.1, 0.8, 0.5), (0.05, 0.02, 0.03), 1.3)], np.float64)
    out = {"mats": mats, "wo": wo, "wi": wi, "u": u}
    for k, m in enumerate(mats):
        f, pdf = ref.bsdf_eval(m, wo, wi)
        swi, sf, spdf, st = ref.bsdf_sample(m, wo, u)
        out.update({f"f{k}": f, f"pdf{k}": pdf, f"swi{k}": swi, f"sf{k}": sf, f"spdf{k}": spdf, f"stype{k}": st})
    np.savez_compressed(os.path.join(HERE, "bsdf_tables_more.npz"), **out)
    sc = scenes.material_room(width=48, height=48)
    for integ, name in (("path", "render_material_room.npz"), ("direct", "render_direct_material_room.npz")):
        S, S2 = ref.scene(sc).render(sc.camera, 48, 48, 1024, 8, seed=29, nthreads=1, integrator=integ)
        bmean, bvar = batch_moments(integ, MATERIAL_BATCHES, 1024, seed0=1000)
        np.savez_compressed(os.path.join(HERE, name), sum=S, sumsq=S2, spp=1024, seed=29, W=48, H=48, max_depth=8,
                            camera=sc.camera, verts=sc.verts, tri_mat=sc.tri_mat, materials=sc.materials,
                            tri_emit=sc.tri_emit, env=np.zeros((0,), np.float32), bmean=bmean, bvar=bvar,
                            batches=MATERIAL_BATCHES, batch_spp=1024)


MATERIAL_BATCHES = 32


def conductors(ref):
    """9. rough conductors of both distributions (Beckmann is the reference's default):
    BSDF tables, and a path render of the conductor room with batch moments."""
    rng = np.random.default_rng(23)
    n = 2000
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    wi = rng.normal(size=(n, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    wi[: n // 2, 2] = np.abs(wi[: n // 2, 2]) * np.sign(wo[: n // 2, 2])   # half on wo's side
    u = rng.random((n, 2))
    mats = np.array([scenes.conductor(0.2, (0.27, 0.68, 1.22), (3.61, 2.63, 2.29), "beckmann"),
                     scenes.conductor(0.05, (1.1, 0.9, 0.6), (2.0, 2.5, 3.0), "beckmann"),
                     scenes.conductor(0.6, (0.2, 0.3, 0.4), (4.0, 3.0, 2.0), "beckmann"),
                     scenes.conductor(0.3, (0.18, 0.42, 1.37), (3.42, 2.35, 1.77), "ggx")], np.float64)
    out = {"mats": mats, "wo": wo, "wi": wi, "u": u}
    for k, m in enumerate(mats):
        f, pdf = ref.bsdf_eval(m, wo, wi)
        swi, sf, spdf, st = ref.bsdf_sample(m, wo, u)
        out.update({f"f{k}": f, f"pdf{k}": pdf, f"swi{k}": swi, f"sf{k}": sf, f"spdf{k}": spdf, f"stype{k}": st})
    np.savez_compressed(os.path.join(HERE, "bsdf_tables_conductor.npz"), **out)
    sc = scenes.conductor_room(width=48, height=48)
    S, S2 = ref.scene(sc).render(sc.camera, 48, 48, 1024, 8, seed=31, nthreads=1)
    bmean, bvar = batch_moments("path", MATERIAL_BATCHES, 1024, seed0=2000, room="conductor")
    np.savez_compressed(os.path.join(HERE, "render_conductor_room.npz"), sum=S, sumsq=S2, spp=1024, seed=31, W=48,
                        H=48, max_depth=8, camera=sc.camera, verts=sc.verts, tri_mat=sc.tri_mat,
                        materials=sc.materials, tri_emit=sc.tri_emit, env=np.zeros((0,), np.float32), bmean=bmean,
                        bvar=bvar, batches=MATERIAL_BATCHES, batch_spp=1024)


def _room(name):
    return (scenes.conductor_room if name == "conductor" else scenes.material_room)(width=48, height=48)


def _material_batch(args):
    integ, spp, seed, room = args
    sc = _room(room)
    S, _ = spo.Oracle("ref").scene(sc).render(sc.camera, 48, 48, spp, 8, seed=seed, nthreads=1, integrator=integ)
    return S / spp


def batch_moments(integ, batches, spp, seed0, room="material"):
    """Per-pixel mean and variance of the mean over independent batches (seeds seed0..).
    Light refracted through the glass box reaches the walls along rare bright paths; the
    per-sample variance of a 1024-sample render under-reads that tail, so the 3-sigma
    comparison uses the spread of batch means instead."""
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(min(batches, os.cpu_count() or 1)) as pool:
        m = np.stack(pool.map(_material_batch, [(integ, spp, seed0 + k, room) for k in range(batches)]))
    return m.mean(0), m.var(0, ddof=1) / batches


if __name__ == "__main__":
    main()
