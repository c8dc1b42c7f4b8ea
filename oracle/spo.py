"""ctypes front-end for the two CPU oracles behind oracle/spo_api.h.

TEST INFRASTRUCTURE ONLY -- imported by tests/, __graft_entry__.smoke() and the
CPU-baseline arm of bench.py, never by the product package.

  Oracle("ref")   oracle/_ref/libspica_ref.so   the reference's own sources, compiled
                                                (only where the reference tree exists)
  Oracle("port")  oracle/_port/libspica_oracle.so  this project's C++ restatement
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout beside this repository (override with SPICA_REFERENCE_SOURCES)
REF_TREE = os.environ.get("SPICA_REFERENCE_SOURCES",
                          os.path.normpath(os.path.join(HERE, "..", "..", "reference", "sources")))
LIBS = {
    "ref": os.path.join(HERE, "_ref", "libspica_ref.so"),
    "port": os.path.join(HERE, "_port", "libspica_oracle.so"),
}

MAT_LAMBERT, MAT_CONDUCTOR, MAT_DIELECTRIC = 0, 1, 2

_dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_bp = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build(kind: str = "port", quiet: bool = True) -> str:
    """Build one oracle library with oracle/Makefile; returns its path."""
    target = {"ref": "ref", "port": "port"}[kind]
    args = ["make", "-C", HERE, "-j", str(os.cpu_count() or 4), target]
    if kind == "ref":
        args.append(f"REF={REF_TREE}")
    out = subprocess.run(args, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"oracle build ({kind}) failed:\n{out.stdout[-4000:]}\n{out.stderr[-4000:]}")
    return LIBS[kind]


def available(kind: str) -> bool:
    return os.path.exists(LIBS[kind])


def _opt(a, dtype):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=dtype)


class Oracle:
    def __init__(self, kind: str = "port"):
        path = LIBS[kind]
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library missing: {path} (run oracle.spo.build('{kind}'))")
        self.kind = kind
        lib = C.CDLL(path)
        lib.spo_scene_create.restype = C.c_void_p
        lib.spo_scene_create.argtypes = [C.c_int, _dp, _ip, C.c_int, _dp, C.c_void_p,
                                         C.c_int, C.c_int, C.c_void_p, C.c_int]
        lib.spo_scene_destroy.argtypes = [C.c_void_p]
        lib.spo_scene_num_lights.argtypes = [C.c_void_p]
        lib.spo_scene_num_lights.restype = C.c_int
        lib.spo_trace.argtypes = [C.c_void_p, C.c_int, C.c_int64, _dp, _dp, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.spo_render.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_int, C.c_uint32, _dp, _dp, C.c_int]
        lib.spo_render_direct.argtypes = lib.spo_render.argtypes
        lib.spo_bsdf_eval.argtypes = [_dp, C.c_int64, _dp, _dp, _dp, _dp]
        lib.spo_bsdf_sample.argtypes = [_dp, C.c_int64, _dp, _dp, _dp, _dp, _dp, _ip]
        lib.spo_name.restype = C.c_char_p
        self.lib = lib

    def name(self) -> str:
        return self.lib.spo_name().decode()

    # ---------------------------------------------------------------- scenes
    def scene(self, sc, use_simd: bool = False) -> "OracleScene":
        return OracleScene(self, sc, use_simd)

    # ---------------------------------------------------------------- BSDFs
    def bsdf_eval(self, mat, wo, wi):
        mat = np.ascontiguousarray(mat, np.float64)
        wo = np.ascontiguousarray(wo, np.float64).reshape(-1, 3)
        wi = np.ascontiguousarray(wi, np.float64).reshape(-1, 3)
        n = wo.shape[0]
        f = np.zeros((n, 3))
        pdf = np.zeros(n)
        self.lib.spo_bsdf_eval(mat, n, wo, wi, f, pdf)
        return f, pdf

    def bsdf_sample(self, mat, wo, u):
        mat = np.ascontiguousarray(mat, np.float64)
        wo = np.ascontiguousarray(wo, np.float64).reshape(-1, 3)
        u = np.ascontiguousarray(u, np.float64).reshape(-1, 2)
        n = wo.shape[0]
        wi = np.zeros((n, 3))
        f = np.zeros((n, 3))
        pdf = np.zeros(n)
        typ = np.zeros(n, np.int32)
        self.lib.spo_bsdf_sample(mat, n, wo, u, wi, f, pdf, typ)
        return wi, f, pdf, typ

    def bsdf_sample_uc(self, mat, wo, u, uc=None):
        """bsdf_sample with the BxDFs' hidden draws visible (the restatement only): with
        uc None the draws come from the hidden generators and are returned per row (NaN
        where a row took none); otherwise row i uses uc[i].  Returns (wi, f, pdf, type,
        uc)."""
        if not hasattr(self.lib, "spo_bsdf_sample_uc"):
            raise NotImplementedError("spo_bsdf_sample_uc is provided by the restatement only")
        fn = self.lib.spo_bsdf_sample_uc
        fn.argtypes = [_dp, C.c_int64, _dp, _dp, C.c_void_p, _dp, _dp, _dp, _ip, _dp]
        mat = np.ascontiguousarray(mat, np.float64)
        wo = np.ascontiguousarray(wo, np.float64).reshape(-1, 3)
        u = np.ascontiguousarray(u, np.float64).reshape(-1, 2)
        n = wo.shape[0]
        wi, f, pdf = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
        typ = np.zeros(n, np.int32)
        uc_in = None if uc is None else np.ascontiguousarray(uc, np.float64).reshape(n)
        uc_out = np.zeros(n)
        fn(mat, n, wo, u, uc_in.ctypes.data if uc_in is not None else None, wi, f, pdf, typ, uc_out)
        return wi, f, pdf, typ, uc_out

    def probe_material(self, mat):
        """The drop-in plugin's material translation on the reference's BSDF for a
        material record (compiled reference only): (record, None) or (None, reason)."""
        mat = np.ascontiguousarray(mat, np.float64)
        rec = np.zeros(8, np.float32)
        why = C.create_string_buffer(256)
        self.lib.spo_probe_material.argtypes = [_dp, C.c_void_p, C.c_char_p, C.c_int]
        rc = self.lib.spo_probe_material(mat, rec.ctypes.data, why, 256)
        return (rec, None) if rc == 0 else (None, why.value.decode())

    # ---------------------------------------------------------------- scene files
    def load_ply(self, path, m16, max_tris=1 << 20):
        """meshio::loadPLY with objectToWorld m16 (row-major 4x4): (n, 9) float64."""
        m = np.ascontiguousarray(m16, np.float64).reshape(16)
        out = np.zeros((max_tris, 9), np.float64)
        n = C.c_int64(0)
        self.lib.spo_load_ply.argtypes = [C.c_char_p, _dp, C.c_int64, C.c_void_p, C.POINTER(C.c_int64)]
        self.lib.spo_load_ply(str(path).encode(), m, max_tris, out.ctypes.data, C.byref(n))
        return out[:min(n.value, max_tris)]

    def transform_chain(self, kinds, params):
        """The scene parser's composition of transform elements (kinds 0 translate,
        1 scale, 2 rotate, 3 lookAt, 4 matrix; 16 parameters each): row-major 4x4."""
        k = np.ascontiguousarray(kinds, np.int32)
        q = np.ascontiguousarray(params, np.float64).reshape(-1)
        out = np.zeros(16, np.float64)
        self.lib.spo_transform_chain.argtypes = [C.c_int, C.c_void_p, _dp, C.c_void_p]
        self.lib.spo_transform_chain(len(k), k.ctypes.data, q, out.ctypes.data)
        return out.reshape(4, 4)

    def load_hdr(self, path, max_pixels=1 << 22):
        """Image::load of a .hdr file: (H, W, 3) float64."""
        out = np.zeros(max_pixels * 3, np.float64)
        w, h = C.c_int(0), C.c_int(0)
        self.lib.spo_load_hdr.argtypes = [C.c_char_p, C.c_int64, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        self.lib.spo_load_hdr(str(path).encode(), max_pixels, out.ctypes.data, C.byref(w), C.byref(h))
        return out[:w.value * h.value * 3].reshape(h.value, w.value, 3)

    # ---------------------------------------------------------------- film output
    # (compiled reference only: the restatement does not carry the image code)
    def _film(self, film):
        film = np.ascontiguousarray(film, np.float32)
        H, W = film.shape[:2]
        return film, W, H

    def film_save_hdr(self, film, path):
        film, W, H = self._film(film)
        self.lib.spo_film_save_hdr.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_char_p]
        self.lib.spo_film_save_hdr(film.ctypes.data, W, H, str(path).encode())

    def film_gamma(self, film, gamma):
        film, W, H = self._film(film)
        out = np.zeros((H, W, 3), np.uint8)
        self.lib.spo_film_gamma.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p]
        self.lib.spo_film_gamma(film.ctypes.data, W, H, gamma, out.ctypes.data)
        return out

    def film_reinhard(self, film, alpha):
        film, W, H = self._film(film)
        out = np.zeros((H, W, 3), np.float64)
        self.lib.spo_film_reinhard.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p]
        self.lib.spo_film_reinhard(film.ctypes.data, W, H, alpha, out.ctypes.data)
        return out

    def triangle_area(self, v):
        v = np.ascontiguousarray(v, np.float64).reshape(9)
        self.lib.spo_triangle_area.restype = C.c_double
        self.lib.spo_triangle_area.argtypes = [C.c_void_p]
        return self.lib.spo_triangle_area(v.ctypes.data)

    def box_intersect(self, lo, hi, org, d, tmax=np.inf):
        """(hit, tnear, tfar) of Bounds3d::intersect."""
        a = [np.ascontiguousarray(x, np.float64).reshape(3) for x in (lo, hi, org, d)]
        tn, tf = C.c_double(np.nan), C.c_double(np.nan)
        self.lib.spo_box_intersect.argtypes = [C.c_void_p] * 4 + [C.c_double, C.c_void_p, C.c_void_p]
        h = self.lib.spo_box_intersect(*[x.ctypes.data for x in a], float(tmax), C.byref(tn), C.byref(tf))
        return bool(h), tn.value, tf.value

    def ray_invdir(self, org, d):
        o = np.ascontiguousarray(org, np.float64).reshape(3)
        dd = np.ascontiguousarray(d, np.float64).reshape(3)
        inv = np.zeros(3, np.float64)
        self.lib.spo_ray_invdir.argtypes = [C.c_void_p] * 3
        self.lib.spo_ray_invdir(o.ctypes.data, dd.ctypes.data, inv.ctypes.data)
        return inv

    def film_drago(self, film, p):
        film, W, H = self._film(film)
        out = np.zeros((H, W, 3), np.float64)
        self.lib.spo_film_drago.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p]
        self.lib.spo_film_drago(film.ctypes.data, W, H, p, out.ctypes.data)
        return out

    def film_durand(self, film, contrast):
        film, W, H = self._film(film)
        out = np.zeros((H, W, 3), np.float64)
        self.lib.spo_film_durand.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p]
        self.lib.spo_film_durand(film.ctypes.data, W, H, contrast, out.ctypes.data)
        return out


class OracleScene:
    """A scene held by one oracle library (see spica_gb300.scenes.Scene for the layout)."""

    def __init__(self, oracle: Oracle, sc, use_simd: bool = False):
        self.o = oracle
        verts = np.ascontiguousarray(sc.verts, np.float64).reshape(-1)
        self._keep = [verts]
        ntri = verts.size // 9
        tri_mat = np.ascontiguousarray(sc.tri_mat, np.int32)
        mats = np.ascontiguousarray(sc.materials, np.float64).reshape(-1)
        emit = _opt(sc.tri_emit, np.float64)
        env = _opt(sc.env, np.float32)
        self._keep += [tri_mat, mats, emit, env]
        env_h, env_w = (env.shape[0], env.shape[1]) if env is not None else (0, 0)
        self.h = oracle.lib.spo_scene_create(
            ntri, verts, tri_mat, mats.size // 8, mats,
            emit.ctypes.data if emit is not None else None,
            env_w, env_h, env.ctypes.data if env is not None else None, int(use_simd))
        if not self.h:
            raise RuntimeError("spo_scene_create failed")
        self.ntri = ntri

    def __del__(self):
        if getattr(self, "h", None):
            self.o.lib.spo_scene_destroy(self.h)
            self.h = None

    def num_lights(self) -> int:
        return self.o.lib.spo_scene_num_lights(self.h)

    def trace(self, org, dir, tmax=None, any_hit=False, nthreads=None):
        org = np.ascontiguousarray(org, np.float64).reshape(-1, 3)
        dir = np.ascontiguousarray(dir, np.float64).reshape(-1, 3)
        n = org.shape[0]
        tm = _opt(tmax, np.float64)
        nthreads = nthreads or os.cpu_count() or 1
        hit = np.zeros(n, np.uint8)
        if any_hit:
            self.o.lib.spo_trace(self.h, 1, n, org, dir, tm.ctypes.data if tm is not None else None,
                                 None, None, hit.ctypes.data, nthreads)
            return hit.astype(bool)
        prim = np.full(n, -1, np.int32)
        t = np.zeros(n)
        self.o.lib.spo_trace(self.h, 0, n, org, dir, tm.ctypes.data if tm is not None else None,
                             prim.ctypes.data, t.ctypes.data, hit.ctypes.data, nthreads)
        return prim, t

    def render(self, cam, W, H, spp, max_depth, seed=0, window=None, nthreads=None, integrator="path"):
        """Per-pixel (sum, sumsq) over spp samples for a film window (fx0, fy0, w, h);
        integrator "path" (PathIntegrator) or "direct" (DirectLightingIntegrator)."""
        fx0, fy0, w, h = window or (0, 0, W, H)
        cam = np.ascontiguousarray(cam, np.float64)
        s = np.zeros((h, w, 3))
        s2 = np.zeros((h, w, 3))
        nthreads = nthreads or os.cpu_count() or 1
        fn = {"path": self.o.lib.spo_render, "direct": self.o.lib.spo_render_direct}[integrator]
        fn(self.h, cam, W, H, fx0, fy0, w, h, spp, max_depth, seed, s, s2, nthreads)
        return s, s2
