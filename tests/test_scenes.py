"""Properties of the seeded procedural workloads (no degenerate triangles, counts,
outward normals of closed meshes, determinism)."""
import numpy as np

from spica_gb300 import scenes


def _areas(v):
    v = v.astype(np.float64)
    return 0.5 * np.linalg.norm(np.cross(v[:, 3:6] - v[:, 0:3], v[:, 6:9] - v[:, 0:3]), axis=1)


def test_box_room():
    sc = scenes.box_room()
    assert sc.ntri == 36 and sc.num_lights == 2
    assert (_areas(sc.verts) > 1e-6).all()
    light = sc.verts[sc.tri_emit[:, 0] > 0].astype(np.float64)
    n = np.cross(light[:, 3:6] - light[:, 0:3], light[:, 6:9] - light[:, 0:3])
    assert (n[:, 1] < 0).all(), "area lights are one-sided: their normal must face the room"


def test_displaced_sphere_exact_count_and_deterministic():
    a = scenes.displaced_sphere(levels=4, seed=0)
    b = scenes.displaced_sphere(levels=4, seed=0)
    assert a.ntri == 4 * 4 ** 4
    assert np.array_equal(a.verts, b.verts)
    assert (_areas(a.verts) > 0).all()
    r = np.linalg.norm(a.verts.reshape(-1, 3), axis=1)
    assert r.min() >= 0.95 - 1e-6 and r.max() <= 1.05 + 1e-6
    # full size: exactly 2^20 triangles (checked on the formula, building it takes ~1 s)
    assert 4 * 4 ** 9 == 1_048_576


def test_outward_normals_of_closed_meshes():
    ms = scenes.mid_scale(n_instances=8, seed=1, sphere_k=3, box_k=2, env_size=(64, 32))
    v = ms.verts[:-10].astype(np.float64)  # instances only (ground + lights at the end)
    n = np.cross(v[:, 3:6] - v[:, 0:3], v[:, 6:9] - v[:, 0:3])
    assert (_areas(ms.verts) > 0).all()
    # every instance is convex: normals point away from its centroid
    for m in np.unique(ms.tri_mat[:-10]):
        sel = ms.tri_mat[:-10] == m
        c = v[sel].reshape(-1, 3).mean(0)
        mid = (v[sel, 0:3] + v[sel, 3:6] + v[sel, 6:9]) / 3
        assert (np.einsum("ij,ij->i", n[sel], mid - c) > 0).all()


def test_microbench_rays():
    sph = scenes.displaced_sphere(levels=3)
    o, d, t = scenes.microbench_rays(sph, 100, 100, 64, 32, seed=1)
    assert o.shape == (200, 3) and d.dtype == np.float32
    assert np.allclose(np.linalg.norm(d.astype(np.float64), axis=1), 1.0, atol=1e-6)
    assert (t[100:] >= 0).all() and (t[100:] <= 2.1).all()


def test_batch_variants_and_guiding_room():
    vs = scenes.batch_variants(64, seed=0)
    assert len(vs) == 64
    assert all(64 <= v.width <= 512 and v.width % 32 == 0 and 16 <= v.spp <= 256 for v in vs)
    gr = scenes.guiding_room()
    assert gr.room_tris == 18 and gr.ntri == 18 + 200 * 12
    assert gr.env is not None and gr.env.max() >= 1.0e4


def test_mid_scale_workload():
    """The 2M-triangle benchmark scene: exact and deterministic triangle count, the
    40 / 40 / 20 material mix and its parameter ranges, four one-sided quad lights facing
    the ground, and the 1024 x 512 sky whose sun carries radiance 1e4 over a 0.5 degree
    disk."""
    sc = scenes.mid_scale()
    again = scenes.mid_scale()
    assert sc.ntri == 2_033_674
    assert np.array_equal(sc.verts, again.verts) and np.array_equal(sc.tri_mat, again.tri_mat)
    assert (_areas(sc.verts) > 1e-9).all()
    m = sc.materials[1:-1]   # the 500 instances (ground first, the lights' black material last)
    kinds = m[:, 0].astype(int)
    frac = np.array([(kinds == k).mean() for k in (scenes.MAT_LAMBERT, scenes.MAT_CONDUCTOR, scenes.MAT_DIELECTRIC)])
    assert len(m) == 500 and np.allclose(frac, [0.4, 0.4, 0.2], atol=0.06), frac
    lam = m[kinds == scenes.MAT_LAMBERT][:, 1:4]
    assert lam.min() >= 0.1 and lam.max() <= 0.9
    emit = sc.tri_emit[:, 0] > 0
    assert emit.sum() == 8 and sc.num_lights == 9   # one area light per triangle, plus the sky
    L = sc.verts[emit].astype(np.float64)
    n = np.cross(L[:, 3:6] - L[:, 0:3], L[:, 6:9] - L[:, 0:3])
    assert (n[:, 2] < 0).all()
    assert sc.env.shape == (512, 1024, 3)
    # sun: the texels above the sky's own maximum hold 1e4 times the solid angle they cover
    H, W = sc.env.shape[:2]
    th = (np.arange(H) + 0.5) / H * np.pi
    texel_sr = (np.pi / H) * (2 * np.pi / W) * np.sin(th)[:, None] * np.ones((1, W))
    excess = np.clip(sc.env[..., 0].astype(np.float64) - 1.0, 0.0, None)
    disk_sr = 2 * np.pi * (1 - np.cos(np.radians(0.25)))
    assert abs((excess * texel_sr).sum() / 1.0e4 - disk_sr) < 0.1 * disk_sr
