"""Seeded procedural scenes for the five benchmark workloads.

A Scene is a flat triangle soup in the layout both the CUDA path (spgpu_upload_scene)
and the CPU oracles take: one material and one optional emission per triangle, as
the reference's scene parser produces for meshes (spica/sceneparser.cc:168-188,
one GeometricPrimitive and one AreaLight per triangle), plus an optional lat-long
environment map whose row 0 is the +z pole (lights/envmap.cc:60-79).

Geometry is generated in float64 with only +, -, *, / and sqrt where exact
reproducibility across hosts matters (the ray-intersection sphere), then rounded to
float32 once; the CPU oracles see the same float32 vertices converted exactly to
float64.  No generated triangle is degenerate (the reference's Triangle
constructor aborts on a zero-area triangle).

Materials use 8-float records: [type, p1..p7]
  0 Lambert      p1..p3 reflectance
  1 GGX conductor p1 alpha (used as is: remapRoughness is off by default,
                 bsdfs/roughconductor.cc:29-36), p2..p4 eta, p5..p7 k
  2 dielectric   p1 interior IOR (exterior 1.0)
A conductor given by its normal-incidence reflectance F0 is stored as eta = 1,
k = 2*sqrt(F0 / (1 - F0)), which gives FrConductor(cos=1) = F0 exactly (F0 <= 0.999).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

MAT_LAMBERT, MAT_CONDUCTOR, MAT_DIELECTRIC, MAT_ROUGH_DIELECTRIC, MAT_PLASTIC = 0, 1, 2, 3, 4
MAT_CONDUCTOR_BECKMANN = 5


@dataclasses.dataclass
class Scene:
    verts: np.ndarray            # (N, 9) float32: p0, p1, p2
    tri_mat: np.ndarray          # (N,) int32
    materials: np.ndarray        # (M, 8) float64
    tri_emit: Optional[np.ndarray] = None   # (N, 3) float32, zero rows = not emitting
    env: Optional[np.ndarray] = None        # (He, We, 3) float32
    camera: Optional[np.ndarray] = None     # eye3, look3, up3, vertical fov (deg)
    width: int = 0
    height: int = 0
    spp: int = 1
    max_depth: int = 8
    name: str = ""

    @property
    def ntri(self) -> int:
        return int(self.verts.shape[0])

    @property
    def num_lights(self) -> int:
        n = 0 if self.tri_emit is None else int(np.count_nonzero(np.any(self.tri_emit != 0, axis=1)))
        return n + (1 if self.env is not None else 0)


def lambert(r, g, b):
    return [MAT_LAMBERT, r, g, b, 0, 0, 0, 0]


def conductor_f0(alpha, f0):
    f0 = np.minimum(np.asarray(f0, np.float64), 0.999)
    k = 2.0 * np.sqrt(f0 / (1.0 - f0))
    return [MAT_CONDUCTOR, alpha, 1.0, 1.0, 1.0, float(k[0]), float(k[1]), float(k[2])]


def conductor(alpha, eta, k, distribution="ggx"):
    """bsdfs/roughconductor.cc with per-channel eta and k; distribution "ggx" or "beckmann"
    (the reference's default)."""
    t = MAT_CONDUCTOR if distribution == "ggx" else MAT_CONDUCTOR_BECKMANN
    return [t, alpha, *eta, *k]


def dielectric(ior):
    return [MAT_DIELECTRIC, ior, 0, 0, 0, 0, 0, 0]


def rough_dielectric(alpha, ior, distribution="beckmann"):
    """bsdfs/roughdielectric.cc with white Kr/Kt; distribution "beckmann" (its default) or "ggx"."""
    return [MAT_ROUGH_DIELECTRIC, alpha, ior, 0.0 if distribution == "beckmann" else 1.0, 0, 0, 0, 0]


def plastic(kd, ks, ior=1.5):
    """bsdfs/plastic.cc: diffuse substrate Kd under a smooth coat with specular Ks."""
    return [MAT_PLASTIC, *kd, *ks, ior]


# ----------------------------------------------------------------------------- helpers
def _quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3); geometric normal = cross(p1-p0, p2-p0)."""
    return [np.r_[p0, p1, p2], np.r_[p0, p2, p3]]


def _box(center, size, angle_deg, axis_up=1):
    """12 triangles of a box rotated about the up axis, outward-facing normals."""
    hx, hy, hz = 0.5 * np.asarray(size, np.float64)
    c = np.asarray(center, np.float64)
    corners = np.array([[sx * hx, sy * hy, sz * hz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)])
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)
    if axis_up == 1:   # rotate about y
        rot = np.array([[ca, 0, sa], [0, 1, 0], [-sa, 0, ca]])
    else:              # rotate about z
        rot = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]])
    P = corners @ rot.T + c
    # faces as corner indices in counter-clockwise order seen from outside
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = []
    for f in faces:
        tris += _quad(P[f[0]], P[f[1]], P[f[2]], P[f[3]])
    out = np.array(tris)
    # make every normal point away from the centre
    n = np.cross(out[:, 3:6] - out[:, 0:3], out[:, 6:9] - out[:, 0:3])
    mid = (out[:, 0:3] + out[:, 3:6] + out[:, 6:9]) / 3.0
    flip = np.einsum("ij,ij->i", n, mid - c) < 0
    out[flip] = out[flip][:, [0, 1, 2, 6, 7, 8, 3, 4, 5]]
    return out


def _grid_tris(A, B, C, k):
    """k*k triangles covering triangle ABC by a barycentric grid (float64, (k*k, 9))."""
    ii, jj = np.meshgrid(np.arange(k + 1), np.arange(k + 1), indexing="ij")
    keep = ii + jj <= k
    idx = -np.ones((k + 1, k + 1), np.int64)
    idx[keep] = np.arange(keep.sum())
    fi, fj = ii[keep].astype(np.float64) / k, jj[keep].astype(np.float64) / k
    P = A[None, :] + (B - A)[None, :] * fi[:, None] + (C - A)[None, :] * fj[:, None]
    i0, j0 = np.meshgrid(np.arange(k), np.arange(k), indexing="ij")
    up = (i0 + j0) <= k - 1
    dn = (i0 + j0) <= k - 2
    t_up = np.stack([idx[i0[up], j0[up]], idx[i0[up] + 1, j0[up]], idx[i0[up], j0[up] + 1]], 1)
    t_dn = np.stack([idx[i0[dn] + 1, j0[dn]], idx[i0[dn] + 1, j0[dn] + 1], idx[i0[dn], j0[dn] + 1]], 1)
    T = np.concatenate([t_up, t_dn])
    return P, T


def _sphere_mesh(seed_polyhedron: str, k: int):
    """Geodesic sphere: each face of the seed split k*k, vertices pushed to the unit sphere.
    Returns (vertices (V,3) float64, triangles (F,3) int64); only +,-,*,/,sqrt are used."""
    if seed_polyhedron == "tetra":
        V = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], np.float64)
        F = [(0, 1, 2), (0, 3, 1), (0, 2, 3), (1, 3, 2)]
    else:  # icosahedron
        g = (1.0 + math.sqrt(5.0)) / 2.0
        V = np.array([[-1, g, 0], [1, g, 0], [-1, -g, 0], [1, -g, 0], [0, -1, g], [0, 1, g],
                      [0, -1, -g], [0, 1, -g], [g, 0, -1], [g, 0, 1], [-g, 0, -1], [-g, 0, 1]], np.float64)
        F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    Ps, Ts, off = [], [], 0
    for (a, b, c) in F:
        P, T = _grid_tris(V[a], V[b], V[c], k)
        Ps.append(P)
        Ts.append(T + off)
        off += P.shape[0]
    P = np.concatenate(Ps)
    T = np.concatenate(Ts)
    P = P / np.sqrt(np.sum(P * P, axis=1, keepdims=True))
    return P, T


def _hash3(ix, iy, iz, seed):
    """Integer lattice hash -> [-1, 1] (uint32 arithmetic, exact on every host)."""
    h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343) ^ iy.astype(np.uint64) * np.uint64(0xD8163841)
         ^ iz.astype(np.uint64) * np.uint64(0xCB1AB31F) ^ np.uint64(seed * 0x9E3779B1 & 0xFFFFFFFF))
    h = h & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    h = (h * np.uint64(0x2C1B3C6D)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(12)
    h = (h * np.uint64(0x297A2D39)) & np.uint64(0xFFFFFFFF)
    h ^= h >> np.uint64(15)
    return (h.astype(np.float64) / 4294967295.0) * 2.0 - 1.0


def value_noise(p, freq, seed):
    """Trilinear value noise with smoothstep fade; p (V,3) float64 -> (V,) in [-1, 1]."""
    q = p * freq + 1024.0
    i = np.floor(q)
    f = q - i
    i = i.astype(np.int64)
    w = f * f * (3.0 - 2.0 * f)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                val = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
                wx = w[:, 0] if dx else 1.0 - w[:, 0]
                wy = w[:, 1] if dy else 1.0 - w[:, 1]
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out += val * wx * wy * wz
    return out


# ----------------------------------------------------------------------------- box room
def box_room(albedo_grey=0.75, albedo_red=(0.63, 0.06, 0.05), albedo_green=(0.14, 0.45, 0.09),
             light_offset=(0.0, 0.0), emission=(17.0, 12.0, 4.0), width=256, height=256, spp=64,
             max_depth=8, name="box_room") -> Scene:
    """Box room: floor, ceiling, back, left (red) and right (green) walls (10 tris), two boxes
    rotated +-17 deg about y (24 tris), one ceiling quad light (2 tris) of 0.25 ceiling width.
    Room [-1,1] x [0,2] x [-1,1], y up, open towards the camera on +z."""
    g = [albedo_grey] * 3 if np.isscalar(albedo_grey) else list(albedo_grey)
    mats = [lambert(*g), lambert(*albedo_red), lambert(*albedo_green)]
    P = lambda x, y, z: np.array([x, y, z], np.float64)  # noqa: E731
    tris, mat = [], []

    def add(ts, m):
        tris.extend(ts)
        mat.extend([m] * len(ts))

    add(_quad(P(-1, 0, -1), P(-1, 0, 1), P(1, 0, 1), P(1, 0, -1)), 0)     # floor
    add(_quad(P(-1, 2, -1), P(1, 2, -1), P(1, 2, 1), P(-1, 2, 1)), 0)     # ceiling
    add(_quad(P(-1, 0, -1), P(1, 0, -1), P(1, 2, -1), P(-1, 2, -1)), 0)   # back
    add(_quad(P(-1, 0, -1), P(-1, 2, -1), P(-1, 2, 1), P(-1, 0, 1)), 1)   # left, red
    add(_quad(P(1, 0, -1), P(1, 0, 1), P(1, 2, 1), P(1, 2, -1)), 2)       # right, green
    add(list(_box((-0.35, 0.6, -0.3), (0.6, 1.2, 0.6), 17.0)), 0)        # tall box
    add(list(_box((0.35, 0.3, 0.35), (0.6, 0.6, 0.6), -17.0)), 0)        # short box
    # light: 0.25 of the ceiling width, just below the ceiling, geometric normal facing down
    cx, cz = light_offset
    h = 0.25
    yl = 2.0 - 1e-3
    light = _quad(P(cx - h, yl, cz - h), P(cx + h, yl, cz - h), P(cx + h, yl, cz + h), P(cx - h, yl, cz + h))
    n0 = np.cross(light[0][3:6] - light[0][0:3], light[0][6:9] - light[0][0:3])
    if n0[1] > 0:
        light = [t[[0, 1, 2, 6, 7, 8, 3, 4, 5]] for t in light]
    nbase = len(tris)
    add(light, 0)
    verts = np.array(tris, np.float64).astype(np.float32)
    emit = np.zeros((verts.shape[0], 3), np.float32)
    emit[nbase:] = emission
    cam = np.array([0.0, 1.0, 3.9, 0.0, 1.0, 0.0, 0.0, 1.0, 0.0, 40.0])
    return Scene(verts, np.array(mat, np.int32), np.array(mats, np.float64), emit, None, cam,
                 width, height, spp, max_depth, name)


def material_room(width=64, height=64, spp=64, max_depth=8, distribution="beckmann") -> Scene:
    """The box room with its tall box a rough dielectric (alpha 0.25, IOR 1.5) and its short
    box plastic (Kd (0.6, 0.3, 0.2), Ks 0.4, IOR 1.5): the remaining reference materials.
    The dielectric box floats 1 cm above the floor: resting on it, its bottom face would be
    coplanar with the floor, and every ray leaving the box downwards would tie between the
    two, a tie that the reference's BVH and the 8-wide one break differently."""
    sc = box_room(width=width, height=height, spp=spp, max_depth=max_depth, name="material_room")
    V = sc.verts.reshape(-1, 3, 3).copy()
    V[10:22, :, 1] += 0.01
    sc.verts = V.reshape(-1, 9).astype(np.float32)
    mats = [list(m) for m in sc.materials] + [rough_dielectric(0.25, 1.5, distribution),
                                              plastic((0.6, 0.3, 0.2), (0.4, 0.4, 0.4), 1.5)]
    tri_mat = sc.tri_mat.copy()
    tri_mat[10:22] = 3   # tall box
    tri_mat[22:34] = 4   # short box
    sc.materials = np.array(mats, np.float64)
    sc.tri_mat = tri_mat
    return sc


def conductor_room(width=64, height=64, spp=64, max_depth=8) -> Scene:
    """The box room with its tall box a rough conductor of the Beckmann distribution (the
    reference's default; alpha 0.2, copper-like eta and k) and its short box a GGX
    conductor (alpha 0.1, gold-like)."""
    sc = box_room(width=width, height=height, spp=spp, max_depth=max_depth, name="conductor_room")
    mats = [list(m) for m in sc.materials] + [
        conductor(0.2, (0.27, 0.68, 1.22), (3.61, 2.63, 2.29), "beckmann"),
        conductor(0.1, (0.18, 0.42, 1.37), (3.42, 2.35, 1.77), "ggx")]
    tri_mat = sc.tri_mat.copy()
    tri_mat[10:22] = len(mats) - 2   # tall box
    tri_mat[22:34] = len(mats) - 1   # short box
    sc.materials = np.array(mats, np.float64)
    sc.tri_mat = tri_mat
    return sc


# ----------------------------------------------------------------------------- ray microbench
def displaced_sphere(levels: int = 9, amplitude: float = 0.05, freq: float = 6.0, seed: int = 0) -> Scene:
    """Geodesic sphere with 4 * 4^levels triangles (levels=9: exactly 1,048,576), radius 1,
    displaced radially by seeded value noise of amplitude `amplitude` * r.  The seed
    polyhedron is the tetrahedron: an icosahedral seed gives 20 * 4^n triangles, which is
    never 2^20."""
    k = 2 ** levels
    P, T = _sphere_mesh("tetra", k)
    r = 1.0 + amplitude * value_noise(P, freq, seed)
    P = P * r[:, None]
    verts = P[T].reshape(-1, 9).astype(np.float32)
    n = verts.shape[0]
    return Scene(verts, np.zeros(n, np.int32), np.array([lambert(0.5, 0.5, 0.5)]), None, None,
                 None, 0, 0, 1, 1, f"displaced_sphere_{n}")


def microbench_rays(sc: Scene, n_coherent: int, n_incoherent: int, width: int = 4096,
                    height: int = 2048, seed: int = 0):
    """Rays of the intersection microbench: n_coherent pinhole rays over a width x height
    raster (pixel centres, strided when n_coherent < width*height) looking at the sphere,
    then n_incoherent rays with origins uniform in the bounding box and directions uniform
    on the sphere.  Returns org (n,3) f32, dir (n,3) f32 (unit), tmax (n,) f32 for any-hit
    (uniform in [0, 2r] for the incoherent half, 2r + distance for the coherent half)."""
    rng = np.random.default_rng(seed)
    v = sc.verts.reshape(-1, 3)
    lo, hi = v.min(0).astype(np.float64), v.max(0).astype(np.float64)
    r = 0.5 * float(np.max(hi - lo))
    # coherent: camera on +z looking at the origin, vertical fov 40 deg
    npix = width * height
    idx = (np.arange(n_coherent, dtype=np.int64) * npix) // max(n_coherent, 1)
    px, py = (idx % width).astype(np.float64) + 0.5, (idx // width).astype(np.float64) + 0.5
    th = math.tan(math.radians(40.0) / 2)
    sx = (2.0 * px / width - 1.0) * th * width / height
    sy = (1.0 - 2.0 * py / height) * th
    d = np.stack([sx, sy, -np.ones_like(sx)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.tile(np.array([0.0, 0.0, 3.2]), (n_coherent, 1))
    # incoherent
    o2 = lo + (hi - lo) * rng.random((n_incoherent, 3))
    z = 2.0 * rng.random(n_incoherent) - 1.0
    ph = 2.0 * math.pi * rng.random(n_incoherent)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    d2 = np.stack([s * np.cos(ph), s * np.sin(ph), z], 1)
    org = np.concatenate([o, o2]).astype(np.float32)
    dir_ = np.concatenate([d, d2]).astype(np.float32)
    # renormalise in float32 so |dir| rounds to 1 as closely as float32 allows
    dir_ = (dir_ / np.sqrt(np.sum(dir_.astype(np.float64) ** 2, 1, keepdims=True))).astype(np.float32)
    tmax = np.concatenate([np.full(n_coherent, 2 * r + 3.2), 2 * r * rng.random(n_incoherent)]).astype(np.float32)
    return org, dir_, tmax


# ----------------------------------------------------------------------------- env maps
def sky_env(width=1024, height=512, sun_dir=(0.55, 0.35, 0.7583), sun_radius_deg=0.25,
            sun_radiance=1.0e4, sky_scale=1.0, horizon=(1.0, 0.95, 0.9), zenith=(0.25, 0.45, 1.0),
            ground=(0.15, 0.13, 0.12)) -> np.ndarray:
    """Procedural lat-long sky, z up: zenith/horizon gradient, dark ground, and a sun disk of
    angular radius sun_radius_deg whose texels carry sun_radiance times their covered
    fraction (8x8 supersampling)."""
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    th = v * math.pi
    ph = u * 2 * math.pi
    cz = np.cos(th)[:, None] * np.ones((1, width))
    t = np.clip(cz, 0.0, 1.0)[..., None]
    sky = (1 - t) * np.array(horizon) + t * np.array(zenith)
    img = np.where((cz > 0)[..., None], sky, np.array(ground)) * sky_scale
    sd = np.asarray(sun_dir, np.float64)
    sd /= np.linalg.norm(sd)
    cos_r = math.cos(math.radians(sun_radius_deg))
    sth, sph = math.acos(sd[2]), math.atan2(sd[1], sd[0]) % (2 * math.pi)
    vi = int(sth / math.pi * height)
    ui = int(sph / (2 * math.pi) * width)
    S = 8
    for y in range(max(0, vi - 3), min(height, vi + 4)):
        for x in range(ui - 3, ui + 4):
            xx = x % width
            sub = (np.arange(S) + 0.5) / S
            tt = (y + sub[:, None]) / height * math.pi
            pp = (xx + sub[None, :]) / width * 2 * math.pi
            dx = np.sin(tt) * np.cos(pp)
            dy = np.sin(tt) * np.sin(pp)
            dz = np.cos(tt) * np.ones_like(pp)
            frac = np.mean(dx * sd[0] + dy * sd[1] + dz * sd[2] >= cos_r)
            if frac > 0:
                img[y, xx] += sun_radiance * frac
    return img.astype(np.float32)


# ----------------------------------------------------------------------------- mid-scale
def mid_scale(n_instances=500, seed=0, width=1920, height=1080, spp=256, max_depth=16,
              sphere_k=16, box_k=16, env_size=(1024, 512)) -> Scene:
    """500 seeded instances of tessellated spheres (icosahedral, 20*k^2 tris) and boxes
    (12*k^2 tris) with scale log-uniform in [0.1, 2] on a ground plane; 40% Lambert
    (albedo U[0.1,0.9]), 40% GGX conductor (alpha U[0.05,0.5], F0 U[0.5,1]), 20% dielectric
    (IOR 1.5); 4 quad area lights and a 1024x512 sky with a 0.5 deg sun of radiance 1e4.
    z up.  With k=16: about 2.06M triangles."""
    rng = np.random.default_rng(seed)
    SP, ST = _sphere_mesh("ico", sphere_k)
    sphere = SP[ST].reshape(-1, 9)
    # tessellated unit box [-1,1]^3: each face a k x k grid of quads
    g = np.linspace(-1.0, 1.0, box_k + 1)
    faces = []
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            a0, a1 = [a for a in range(3) if a != axis]
            for i in range(box_k):
                for j in range(box_k):
                    q = np.zeros((4, 3))
                    for c, (di, dj) in enumerate([(0, 0), (1, 0), (1, 1), (0, 1)]):
                        q[c, axis] = sgn
                        q[c, a0] = g[i + di]
                        q[c, a1] = g[j + dj]
                    faces += _quad(q[0], q[1], q[2], q[3])
    box = np.array(faces)
    n = np.cross(box[:, 3:6] - box[:, 0:3], box[:, 6:9] - box[:, 0:3])
    mid = (box[:, 0:3] + box[:, 3:6] + box[:, 6:9]) / 3.0
    flip = np.einsum("ij,ij->i", n, mid) < 0
    box[flip] = box[flip][:, [0, 1, 2, 6, 7, 8, 3, 4, 5]]

    extent = 40.0
    mats, tris, tmat = [], [], []
    mats.append(lambert(0.5, 0.5, 0.5))  # ground
    for i in range(n_instances):
        kind = rng.random()
        scale = 0.1 * (20.0 ** rng.random())
        cx, cy = (rng.random(2) * 2 - 1) * extent
        m = rng.random()
        if m < 0.4:
            mats.append(lambert(*(0.1 + 0.8 * rng.random(3))))
        elif m < 0.8:
            mats.append(conductor_f0(0.05 + 0.45 * rng.random(), 0.5 + 0.5 * rng.random(3)))
        else:
            mats.append(dielectric(1.5))
        mid_ = len(mats) - 1
        if kind < 0.5:
            t = sphere.copy().reshape(-1, 3) * scale + np.array([cx, cy, scale])
        else:
            a = rng.random() * math.pi
            ca, sa = math.cos(a), math.sin(a)
            R = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]])
            t = (box.reshape(-1, 3) * scale) @ R.T + np.array([cx, cy, scale])
        t = t.reshape(-1, 9)
        tris.append(t)
        tmat.append(np.full(t.shape[0], mid_, np.int32))
    G = 1.6 * extent
    ground = np.array(_quad(np.array([-G, -G, 0.0]), np.array([G, -G, 0.0]), np.array([G, G, 0.0]),
                            np.array([-G, G, 0.0])))
    tris.append(ground)
    tmat.append(np.zeros(2, np.int32))
    # 4 quad area lights facing down
    lights = []
    for (lx, ly) in [(-15, -15), (15, -15), (-15, 15), (15, 15)]:
        h = 2.0
        z = 12.0
        q = _quad(np.array([lx - h, ly - h, z]), np.array([lx - h, ly + h, z]), np.array([lx + h, ly + h, z]),
                  np.array([lx + h, ly - h, z]))
        nn = np.cross(q[0][3:6] - q[0][0:3], q[0][6:9] - q[0][0:3])
        if nn[2] > 0:
            q = [tq[[0, 1, 2, 6, 7, 8, 3, 4, 5]] for tq in q]
        lights += q
    mats.append(lambert(0.0, 0.0, 0.0))
    nl = len(lights)
    tris.append(np.array(lights))
    tmat.append(np.full(nl, len(mats) - 1, np.int32))
    verts = np.concatenate(tris).astype(np.float32)
    tri_mat = np.concatenate(tmat)
    emit = np.zeros((verts.shape[0], 3), np.float32)
    emit[-nl:] = (40.0, 38.0, 35.0)
    env = sky_env(env_size[0], env_size[1])
    cam = np.array([0.0, -58.0, 16.0, 0.0, 0.0, 1.5, 0.0, 0.0, 1.0, 50.0])
    return Scene(verts, tri_mat, np.array(mats, np.float64), emit, env, cam, width, height, spp,
                 max_depth, "mid_scale")


# ----------------------------------------------------------------------------- batched
def batch_variants(count=64, seed=0, max_depth=8):
    """Seeded variants of the box room: square resolution in {64..512} step 32, spp in
    {16..256}, wall albedos U[0.1,0.9], light centre jittered by up to 20% of the ceiling."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        res = int(rng.integers(2, 17)) * 32
        spp = int(rng.integers(16, 257))
        grey = float(0.1 + 0.8 * rng.random())
        red = tuple(float(x) for x in 0.1 + 0.8 * rng.random(3))
        green = tuple(float(x) for x in 0.1 + 0.8 * rng.random(3))
        off = tuple(float(x) for x in (rng.random(2) * 2 - 1) * 0.2 * 2.0 * 0.5)
        out.append(box_room(grey, red, green, off, width=res, height=res, spp=spp, max_depth=max_depth,
                            name=f"variant_{i}"))
    return out


# ----------------------------------------------------------------------------- guiding room
def guiding_room(n_boxes=200, seed=0, width=1280, height=720, spp=64, max_depth=12) -> Scene:
    """Closed 10 x 8 x 4 room (z up, Lambert 0.7) whose +y wall has one 0.5 x 0.5 window;
    outside, a sky of radiance 1 with a 0.5 deg sun of radiance 1e5 shining in through the
    window; 200 seeded boxes (12 tris each) on the floor.  The window wall is triangulated
    around the opening, so the room has 18 triangles rather than 12."""
    rng = np.random.default_rng(seed)
    X, Y, Z = 10.0, 8.0, 4.0
    P = lambda x, y, z: np.array([x, y, z], np.float64)  # noqa: E731
    tris = []
    tris += _quad(P(0, 0, 0), P(0, Y, 0), P(X, Y, 0), P(X, 0, 0))        # floor (normal +z)
    tris += _quad(P(0, 0, Z), P(X, 0, Z), P(X, Y, Z), P(0, Y, Z))        # ceiling
    tris += _quad(P(0, 0, 0), P(X, 0, 0), P(X, 0, Z), P(0, 0, Z))        # y = 0 wall
    tris += _quad(P(0, 0, 0), P(0, 0, Z), P(0, Y, Z), P(0, Y, 0))        # x = 0 wall
    tris += _quad(P(X, 0, 0), P(X, Y, 0), P(X, Y, Z), P(X, 0, Z))        # x = X wall
    # y = Y wall with a window [wx0, wx1] x [wz0, wz1]
    wx0, wx1, wz0, wz1 = 6.5, 7.0, 2.5, 3.0
    for (a0, a1, b0, b1) in [(0, wx0, 0, Z), (wx1, X, 0, Z), (wx0, wx1, 0, wz0), (wx0, wx1, wz1, Z)]:
        tris += _quad(P(a0, Y, b0), P(a0, Y, b1), P(a1, Y, b1), P(a1, Y, b0))
    nroom = len(tris)
    for _ in range(n_boxes):
        s = 0.2 + 0.6 * rng.random(3)
        s[2] = 0.2 + 1.2 * rng.random()
        c = (0.5 + (X - 1) * rng.random(), 0.5 + (Y - 1.5) * rng.random(), 0.5 * s[2])
        tris += list(_box(c, s, 360 * rng.random(), axis_up=2))
    verts = np.array(tris, np.float64).astype(np.float32)
    mats = np.array([lambert(0.7, 0.7, 0.7)], np.float64)
    sun = np.array([0.25, 0.8, 0.35])
    env = sky_env(1024, 512, sun_dir=sun / np.linalg.norm(sun), sun_radiance=1.0e5,
                  horizon=(1.0, 1.0, 1.0), zenith=(1.0, 1.0, 1.0), ground=(1.0, 1.0, 1.0))
    cam = np.array([1.0, 1.0, 2.2, 7.0, 6.0, 1.2, 0.0, 0.0, 1.0, 60.0])
    sc = Scene(verts, np.zeros(verts.shape[0], np.int32), mats, None, env, cam, width, height, spp,
               max_depth, "guiding_room")
    sc.room_tris = nroom
    return sc
