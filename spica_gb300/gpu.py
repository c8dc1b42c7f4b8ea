"""Host-side mirror of the reference's accelerator and integrator plugins over the
C ABI of libspica_gpu.so (include/spica_gpu.h), through ctypes.

Names follow the reference's interfaces:
  GpuBVHAccel       -- Accelerator (core/accelerator.h:23): construct(), worldBound(),
                       intersect(...) for closest hit and any hit
                       (BVHAccel::intersect, accelerators/bvh.cc:315-329)
  GpuPathIntegrator -- SamplerIntegrator/PathIntegrator (core/integrator.h:44,
                       integrators/path/path.h:21): render(camera, scene, params)
                       reading "maxDepth" and "sampleCount" like the reference
                       (core/integrator.cc:63, integrators/path/path.cc:68)
Errors: every negative status of the C ABI raises SpgpuError with the library's
message (the reference aborts via Assertion/FatalError, core/common.h:69-115).
The CUDA library is required: there is no CPU fallback; loading fails loudly when
the extension has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB


class SpgpuError(RuntimeError):
    pass


class BVHInfo(C.Structure):
    _fields_ = [("triangles", C.c_int64), ("wide_nodes", C.c_int64), ("depth", C.c_int32),
                ("lights", C.c_int32), ("build_ms", C.c_double), ("bounds", C.c_float * 6)]


class TraceCounters(C.Structure):
    _fields_ = [("rays", C.c_int64), ("nodes_per_ray", C.c_double), ("tris_per_ray", C.c_double)]


class RenderDesc(C.Structure):
    _fields_ = [("camera", C.c_float * 10), ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
                ("sample_offset", C.c_int32), ("max_depth", C.c_int32), ("seed", C.c_uint32),
                ("integrator", C.c_int32), ("reserved", C.c_int32 * 3)]


class RenderStats(C.Structure):
    _fields_ = [("paths", C.c_int64), ("rays_closest", C.c_int64), ("rays_shadow", C.c_int64), ("ms", C.c_double),
                ("kernel_launches", C.c_int64)]


class KernelProfile(C.Structure):
    _fields_ = [("kernel_ms", C.c_double * 8), ("launches", C.c_int64 * 8), ("paths", C.c_int64),
                ("rays_closest", C.c_int64), ("rays_shadow", C.c_int64), ("closest_nodes_per_ray", C.c_double),
                ("closest_tris_per_ray", C.c_double), ("shadow_nodes_per_ray", C.c_double),
                ("shadow_tris_per_ray", C.c_double)]


KERNEL_CLASSES = ["raygen", "extend", "shade_lambert", "shade_conductor", "shade_dielectric", "shadow", "finish"]


class BatchItem(C.Structure):
    _fields_ = [("ntri", C.c_int32), ("verts", C.c_void_p), ("tri_mat", C.c_void_p), ("nmat", C.c_int32),
                ("materials", C.c_void_p), ("tri_emit", C.c_void_p), ("desc", RenderDesc)]


class BatchTuning(C.Structure):
    _fields_ = [("block", C.c_int32), ("tile_pixels", C.c_int32), ("chunk_spp", C.c_int32),
                ("candidates", C.c_int32), ("calib_ms", C.c_double), ("engine", C.c_int32),
                ("pool_slots", C.c_int32), ("pool_lanes", C.c_int32), ("iterations", C.c_int32)]


class GuidingConfig(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("bsdf_fraction", C.c_float), ("batch", C.c_int32),
                ("seed", C.c_uint32), ("capacity", C.c_int32), ("fault_injection", C.c_int32),
                ("guided_bounces", C.c_int32), ("reserved", C.c_int32 * 1)]


GUIDE_GUIDED, GUIDE_COLLECT, GUIDE_MEGAKERNEL = 1, 2, 4
BATCH_STREAM, BATCH_PERSISTENT = 1, 2   # batch engines (spgpu_batch_tuning.engine)
FILM_RGBE, FILM_GAMMA_BYTES, FILM_REINHARD, FILM_DRAGO, FILM_DURAND = 0, 1, 2, 3, 4


def film_resolve(ctx: "Context", film_dev, fmt: int, param: float = 0.0, stream: int = 0):
    """spgpu_film_resolve of a device film (torch (H, W, 4) float32): RGBE bytes (H, W, 4),
    gamma-corrected bytes (H, W, 3), or a Reinhard-, Drago- or Durand-mapped image
    (H, W, 3) float32, on the device."""
    import torch
    H, W = int(film_dev.shape[0]), int(film_dev.shape[1])
    if fmt == FILM_RGBE:
        out = torch.empty((H, W, 4), dtype=torch.uint8, device=film_dev.device)
    elif fmt == FILM_GAMMA_BYTES:
        out = torch.empty((H, W, 3), dtype=torch.uint8, device=film_dev.device)
    else:
        out = torch.empty((H, W, 3), dtype=torch.float32, device=film_dev.device)
    _check(ctx.lib.spgpu_film_resolve(ctx.h, _ptr(film_dev), W, H, fmt, float(param), _ptr(out),
                                      C.c_void_p(stream) if stream else None), "spgpu_film_resolve")
    return out


def write_hdr(path: str, rgbe) -> None:
    """spgpu_write_hdr: (H, W, 4) uint8 RGBE pixels to a Radiance .hdr file laid out as
    the reference's Image::saveHdr writes it."""
    a = np.ascontiguousarray(rgbe, np.uint8)
    _check(load_library().spgpu_write_hdr(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0]),
           "spgpu_write_hdr")


class SceneFile(C.Structure):
    _fields_ = [("ntri", C.c_int32), ("verts", C.c_void_p), ("tri_mat", C.c_void_p), ("nmat", C.c_int32),
                ("materials", C.c_void_p), ("tri_emit", C.c_void_p), ("env_width", C.c_int32),
                ("env_height", C.c_int32), ("env", C.c_void_p), ("desc", RenderDesc), ("internal", C.c_void_p)]


def load_scene(path: str):
    """spgpu_scene_load: a scene file of the reference's XML format (SceneParser,
    spica/sceneparser.cc) as a scenes.Scene (arrays copied out) plus the integrator
    ("path" or "direct")."""
    from .scenes import Scene
    lib = load_library()
    out = C.POINTER(SceneFile)()
    _check(lib.spgpu_scene_load(str(path).encode(), C.byref(out)), "spgpu_scene_load")
    try:
        f = out.contents
        n, m = f.ntri, f.nmat

        def arr(ptr, count, dtype):
            if count == 0:
                return np.zeros((0,), dtype)
            ct = {np.float32: C.c_float, np.int32: C.c_int32}[dtype]
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(count,)).copy()

        env = None
        if f.env:
            env = arr(f.env, f.env_width * f.env_height * 3, np.float32).reshape(f.env_height, f.env_width, 3)
        d = f.desc
        sc = Scene(verts=arr(f.verts, 9 * n, np.float32).reshape(n, 9), tri_mat=arr(f.tri_mat, n, np.int32),
                   materials=arr(f.materials, 8 * m, np.float32).reshape(m, 8).astype(np.float64),
                   tri_emit=arr(f.tri_emit, 3 * n, np.float32).reshape(n, 3), env=env,
                   camera=np.array(list(d.camera), np.float32), width=d.width, height=d.height, spp=d.spp,
                   max_depth=d.max_depth, name=os.path.basename(str(path)))
        integrator = "direct" if d.integrator == 1 else "path"
    finally:
        lib.spgpu_scene_free(out)
    return sc, integrator


def load_hdr(path: str) -> np.ndarray:
    """spgpu_load_hdr: a Radiance .hdr file as (H, W, 3) float32, as the reference's
    Image::loadHdr reads it."""
    lib = load_library()
    w, h = C.c_int32(0), C.c_int32(0)
    _check(lib.spgpu_load_hdr(str(path).encode(), None, 0, C.byref(w), C.byref(h)), "spgpu_load_hdr")
    out = np.zeros((h.value, w.value, 3), np.float32)
    _check(lib.spgpu_load_hdr(str(path).encode(), out.ctypes.data, w.value * h.value, C.byref(w), C.byref(h)),
           "spgpu_load_hdr")
    return out


def write_png(path: str, rgb) -> None:
    """spgpu_write_png: (H, W, 3) uint8 pixels to an 8-bit RGB PNG."""
    a = np.ascontiguousarray(rgb, np.uint8)
    _check(load_library().spgpu_write_png(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0]),
           "spgpu_write_png")
GUIDE_PARAMS = 11560


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("pass_lanes", C.c_int), ("wavefront", C.c_int), ("reserved", C.c_int * 5)]


# every extern "C" symbol include/spica_gpu.h declares
EXPORTS = ["spgpu_create", "spgpu_destroy", "spgpu_last_error", "spgpu_version", "spgpu_upload_scene",
           "spgpu_build_bvh", "spgpu_bvh_stats", "spgpu_trace", "spgpu_trace_host", "spgpu_trace_stats",
           "spgpu_trace_host_noalloc", "spgpu_film_resolve", "spgpu_write_hdr", "spgpu_write_png",
           "spgpu_render", "spgpu_render_host", "spgpu_render_profile", "spgpu_batch_prepare",
           "spgpu_batch_film_pixels", "spgpu_batch_run", "spgpu_guiding_init", "spgpu_guiding_render",
           "spgpu_guiding_train", "spgpu_guiding_samples", "spgpu_guiding_ring", "spgpu_guiding_params", "spgpu_guiding_mlp",
           "spgpu_guiding_grad", "spgpu_scene_load", "spgpu_scene_free", "spgpu_load_hdr", "spgpu_bsdf_eval",
           "spgpu_bsdf_sample", "spgpu_sampler_generate", "spgpu_batch_profile"]

_lib = None


def load_library(path: Optional[str] = None):
    """Load libspica_gpu.so (built by spica_gb300.build).  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise SpgpuError(f"CUDA library not built: {p} (run python -m spica_gb300.build)")
    lib = C.CDLL(p)
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
    lib.spgpu_create.argtypes = [C.POINTER(Config), C.POINTER(vp)]
    lib.spgpu_destroy.argtypes = [vp]
    lib.spgpu_destroy.restype = None
    lib.spgpu_last_error.restype = C.c_char_p
    lib.spgpu_version.restype = C.c_char_p
    lib.spgpu_upload_scene.argtypes = [vp, i32, vp, vp, i32, vp, vp, i32, i32, vp]
    lib.spgpu_build_bvh.argtypes = [vp]
    lib.spgpu_bvh_stats.argtypes = [vp, C.POINTER(BVHInfo)]
    lib.spgpu_trace.argtypes = [vp, C.c_int, vp, vp, i64, vp, vp]
    lib.spgpu_trace_host.argtypes = [vp, C.c_int, vp, vp, i64, vp]
    lib.spgpu_trace_host_noalloc.argtypes = [vp, C.c_int, vp, vp, i64, vp]
    lib.spgpu_film_resolve.argtypes = [vp, vp, i32, i32, i32, C.c_double, vp, vp]
    lib.spgpu_write_hdr.argtypes = [C.c_char_p, vp, i32, i32]
    lib.spgpu_write_png.argtypes = [C.c_char_p, vp, i32, i32]
    lib.spgpu_scene_load.argtypes = [C.c_char_p, C.POINTER(C.POINTER(SceneFile))]
    lib.spgpu_scene_free.argtypes = [C.POINTER(SceneFile)]
    lib.spgpu_scene_free.restype = None
    lib.spgpu_load_hdr.argtypes = [C.c_char_p, vp, i32, C.POINTER(i32), C.POINTER(i32)]
    lib.spgpu_trace_stats.argtypes = [vp, C.c_int, vp, vp, i64, vp, C.POINTER(TraceCounters)]
    lib.spgpu_render.argtypes = [vp, C.POINTER(RenderDesc), vp, C.POINTER(RenderStats), vp]
    lib.spgpu_render_host.argtypes = [vp, C.POINTER(RenderDesc), vp, C.POINTER(RenderStats)]
    lib.spgpu_render_profile.argtypes = [vp, C.POINTER(RenderDesc), vp, C.POINTER(KernelProfile), vp]
    lib.spgpu_batch_prepare.argtypes = [vp, i32, C.POINTER(BatchItem), i32, C.POINTER(BatchTuning)]
    lib.spgpu_batch_film_pixels.argtypes = [vp]
    lib.spgpu_batch_run.argtypes = [vp, vp, vp, C.POINTER(RenderStats), vp]
    lib.spgpu_batch_profile.argtypes = [vp, vp, C.POINTER(KernelProfile), vp]
    lib.spgpu_guiding_init.argtypes = [vp, C.POINTER(GuidingConfig)]
    lib.spgpu_guiding_render.argtypes = [vp, C.POINTER(RenderDesc), vp, i32, C.POINTER(RenderStats), vp]
    lib.spgpu_guiding_train.argtypes = [vp, i32, C.POINTER(C.c_double)]
    lib.spgpu_guiding_samples.argtypes = [vp]
    lib.spgpu_guiding_ring.argtypes = [vp, vp, i32, C.POINTER(i32)]
    lib.spgpu_guiding_params.argtypes = [vp, vp, i32]
    lib.spgpu_guiding_mlp.argtypes = [vp, vp, i32, vp, vp]
    lib.spgpu_guiding_grad.argtypes = [vp, vp, i32, vp, C.POINTER(C.c_double), vp]
    lib.spgpu_bsdf_eval.argtypes = [vp, vp, i64, vp, vp, vp, vp]
    lib.spgpu_bsdf_sample.argtypes = [vp, vp, i64, vp, vp, vp, vp, vp, vp]
    lib.spgpu_sampler_generate.argtypes = [vp, i64, vp, vp, vp, vp]
    for name in EXPORTS:
        if name not in ("spgpu_destroy", "spgpu_last_error", "spgpu_version"):
            getattr(lib, name).restype = C.c_int
    lib.spgpu_batch_film_pixels.restype = C.c_int64
    lib.spgpu_guiding_samples.restype = C.c_int64
    if path is None:
        _lib = lib
    return lib


def _check(rc: int, what: str):
    if rc != 0:
        # the message may quote bytes of a malformed input file
        msg = _lib.spgpu_last_error().decode("utf-8", "replace") if _lib is not None else ""
        raise SpgpuError(f"{what} failed ({rc}): {msg}")


def _ptr(a) -> int:
    """Device or host address of a torch tensor or numpy array."""
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class Context:
    """One device, one scene and its BVH (spgpu_ctx)."""

    def __init__(self, device: int = 0, pass_lanes: int = 0, wavefront: int = 0):
        self.lib = load_library()
        cfg = Config(device=device, pass_lanes=pass_lanes, wavefront=wavefront)
        h = C.c_void_p()
        _check(self.lib.spgpu_create(C.byref(cfg), C.byref(h)), "spgpu_create")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.spgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def upload_scene(self, sc):
        verts = np.ascontiguousarray(sc.verts, np.float32)
        tri_mat = np.ascontiguousarray(sc.tri_mat, np.int32)
        mats = np.ascontiguousarray(sc.materials, np.float32)
        emit = None if sc.tri_emit is None else np.ascontiguousarray(sc.tri_emit, np.float32)
        env = None if sc.env is None else np.ascontiguousarray(sc.env, np.float32)
        eh, ew = (env.shape[0], env.shape[1]) if env is not None else (0, 0)
        _check(self.lib.spgpu_upload_scene(self.h, verts.shape[0], verts.ctypes.data, tri_mat.ctypes.data,
                                           mats.shape[0], mats.ctypes.data,
                                           emit.ctypes.data if emit is not None else None, ew, eh,
                                           env.ctypes.data if env is not None else None), "spgpu_upload_scene")

    def build_bvh(self):
        _check(self.lib.spgpu_build_bvh(self.h), "spgpu_build_bvh")

    def bvh_info(self) -> BVHInfo:
        info = BVHInfo()
        _check(self.lib.spgpu_bvh_stats(self.h, C.byref(info)), "spgpu_bvh_stats")
        return info


class GpuBVHAccel:
    """Accelerator over the device-built compressed 8-wide BVH."""

    def __init__(self, scene, device: int = 0, ctx: Optional[Context] = None):
        self.ctx = ctx or Context(device)
        self.scene = scene
        self.ctx.upload_scene(scene)
        self.constructed = False

    def construct(self):
        self.ctx.build_bvh()
        self.constructed = True
        return self

    def worldBound(self):
        b = self.ctx.bvh_info().bounds
        return np.array(b[0:3]), np.array(b[3:6])

    def info(self) -> BVHInfo:
        return self.ctx.bvh_info()

    # --- device tensors (torch): org_tmin, dir_tmax (n, 4) float32 on the GPU
    def intersect_device(self, org_tmin, dir_tmax, out, any_hit: bool = False, stream: int = 0):
        n = org_tmin.shape[0]
        _check(self.ctx.lib.spgpu_trace(self.ctx.h, int(any_hit), _ptr(org_tmin), _ptr(dir_tmax), n, _ptr(out),
                                        C.c_void_p(stream) if stream else None), "spgpu_trace")

    def intersect_stats(self, org_tmin, dir_tmax, out, any_hit: bool = False) -> TraceCounters:
        c = TraceCounters()
        _check(self.ctx.lib.spgpu_trace_stats(self.ctx.h, int(any_hit), _ptr(org_tmin), _ptr(dir_tmax),
                                              org_tmin.shape[0], _ptr(out), C.byref(c)), "spgpu_trace_stats")
        return c

    # --- host arrays (numpy)
    def intersect(self, org, dir, tmax=None, tmin=None):
        """Closest hit for n rays: returns (prim (n,) int32, -1 = miss; t; u; v)."""
        ot, dt = _pack_rays(org, dir, tmax, tmin)
        out = np.zeros((ot.shape[0], 4), np.float32)
        _check(self.ctx.lib.spgpu_trace_host(self.ctx.h, 0, ot.ctypes.data, dt.ctypes.data, ot.shape[0],
                                             out.ctypes.data), "spgpu_trace_host")
        prim = out[:, 1].view(np.int32).copy()
        return prim, out[:, 0].copy(), out[:, 2].copy(), out[:, 3].copy()

    def intersect_any(self, org, dir, tmax=None, tmin=None):
        """Any hit in (eps, tmax] for n rays: returns (n,) bool."""
        ot, dt = _pack_rays(org, dir, tmax, tmin)
        out = np.zeros(ot.shape[0], np.uint32)
        _check(self.ctx.lib.spgpu_trace_host(self.ctx.h, 1, ot.ctypes.data, dt.ctypes.data, ot.shape[0],
                                             out.ctypes.data), "spgpu_trace_host")
        return out.astype(bool)

    NOALLOC_MAX_RAYS = 65536

    def intersect_noalloc(self, org, dir, tmax=None, tmin=None, any_hit=False):
        """intersect / intersect_any through spgpu_trace_host_noalloc (no device
        allocation; at most NOALLOC_MAX_RAYS rays per call)."""
        ot, dt = _pack_rays(org, dir, tmax, tmin)
        out = np.zeros(ot.shape[0], np.uint32) if any_hit else np.zeros((ot.shape[0], 4), np.float32)
        _check(self.ctx.lib.spgpu_trace_host_noalloc(self.ctx.h, 1 if any_hit else 0, ot.ctypes.data, dt.ctypes.data,
                                                     ot.shape[0], out.ctypes.data), "spgpu_trace_host_noalloc")
        if any_hit:
            return out.astype(bool)
        prim = out[:, 1].view(np.int32).copy()
        return prim, out[:, 0].copy(), out[:, 2].copy(), out[:, 3].copy()


def _pack_rays(org, dir, tmax=None, tmin=None):
    org = np.asarray(org, np.float32).reshape(-1, 3)
    dir = np.asarray(dir, np.float32).reshape(-1, 3)
    n = org.shape[0]
    ot = np.empty((n, 4), np.float32)
    dt = np.empty((n, 4), np.float32)
    ot[:, :3] = org
    ot[:, 3] = 0.0 if tmin is None else tmin
    dt[:, :3] = dir
    dt[:, 3] = 1.0e32 if tmax is None else tmax
    return ot, dt


class GpuBSDF:
    """One material's BSDF on the device, function by function (spgpu_bsdf_eval /
    spgpu_bsdf_sample): BSDF::f, BSDF::pdf and BSDF::sample (core/bsdf.cc:49-136) in
    the shading frame (z = shading normal).  material: 8-float SPGPU_MAT_* record."""

    def __init__(self, material, ctx: Optional[Context] = None, device: int = 0):
        self.ctx = ctx or Context(device)
        self.material = np.ascontiguousarray(material, np.float32).reshape(8)

    def f_pdf(self, wo, wi):
        """(f (n, 3), pdf (n,)) for directions wo, wi (n, 3)."""
        wo = np.ascontiguousarray(wo, np.float32).reshape(-1, 3)
        wi = np.ascontiguousarray(wi, np.float32).reshape(-1, 3)
        n = wo.shape[0]
        f = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        _check(self.ctx.lib.spgpu_bsdf_eval(self.ctx.h, self.material.ctypes.data, n, wo.ctypes.data, wi.ctypes.data,
                                            f.ctypes.data, pdf.ctypes.data), "spgpu_bsdf_eval")
        return f, pdf

    def sample(self, wo, u):
        """BSDF::sample for directions wo (n, 3) and numbers u (n, 3): the 2D sample and
        the draw the reference's rough dielectric and plastic take from their own
        generator.  Returns (wi, f, pdf, type)."""
        wo = np.ascontiguousarray(wo, np.float32).reshape(-1, 3)
        u = np.ascontiguousarray(u, np.float32).reshape(-1, 3)
        n = wo.shape[0]
        wi = np.zeros((n, 3), np.float32)
        f = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        t = np.zeros(n, np.int32)
        _check(self.ctx.lib.spgpu_bsdf_sample(self.ctx.h, self.material.ctypes.data, n, wo.ctypes.data, u.ctypes.data,
                                              wi.ctypes.data, f.ctypes.data, pdf.ctypes.data, t.ctypes.data),
               "spgpu_bsdf_sample")
        return wi, f, pdf, t


def philox(counter, key, ctx: Optional[Context] = None):
    """Philox4x32-10 on the device (spgpu_sampler_generate): counter (n, 4) and key (n, 2)
    uint32 -> (raw words (n, 4) uint32, uniforms (n, 4) float32 in [0, 1))."""
    ctx = ctx or Context()
    c = np.ascontiguousarray(counter, np.uint32).reshape(-1, 4)
    k = np.ascontiguousarray(key, np.uint32).reshape(-1, 2)
    if c.shape[0] != k.shape[0]:
        raise ValueError("counter and key need the same number of rows")
    raw = np.zeros_like(c)
    u = np.zeros(c.shape, np.float32)
    _check(ctx.lib.spgpu_sampler_generate(ctx.h, c.shape[0], c.ctypes.data, k.ctypes.data, raw.ctypes.data,
                                          u.ctypes.data), "spgpu_sampler_generate")
    return raw, u


CAMERA_BOUNCE = 0xFFFF   # the bounce word of the camera ray's counter
STREAM_TAG = 0x5350      # the fourth counter word of every renderer draw


class GpuSampler:
    """The renderer's random numbers behind the reference's Sampler interface
    (core/sampler.h:24-37: startPixel, startNextSample, get1D, get2D, clone).  The
    reference's Independent sampler (samplers/independent.cc:6-23) reads one MT19937
    stream per thread; here every (seed, film pixel, sample index) has its own
    Philox4x32-10 stream, so a pixel's numbers do not depend on which thread draws them.
    Dimensions run in the renderer's order: dimensions 0-3 are the camera block
    (bounce word 0xFFFF, stream 0: film x, film y, then two unused lens numbers), and
    dimension 4 + k is lane k % 4 of stream (k // 4) % 4 at bounce k // 16."""

    BLOCKS = 16   # counter blocks fetched per device call

    def __init__(self, seed: int = 0, ctx: Optional[Context] = None, width: Optional[int] = None):
        self.seed = int(seed) & 0xFFFFFFFF
        self.ctx = ctx
        self.width = width
        self.pixel = 0
        self.sample = -1
        self.dim = 0
        self._cache = {}

    def clone(self, seed: int) -> "GpuSampler":
        return GpuSampler(seed, ctx=self.ctx, width=self.width)

    def startPixel(self, x: int, y: int = 0):
        """Select the film pixel (x, y) of a film `width` wide (the key is the film's pixel
        index y * width + x); with no width, x is the film pixel index itself."""
        self.pixel = int(y) * int(self.width) + int(x) if self.width else int(x)
        self.sample = -1
        self.dim = 0
        self._cache = {}

    def startNextSample(self):
        self.sample += 1
        self.dim = 0
        self._cache = {}

    @staticmethod
    def block_of(dim: int):
        """(bounce word, stream, lane) of a dimension."""
        if dim < 4:
            return CAMERA_BOUNCE, 0, dim
        k = dim - 4
        return k // 16, (k // 4) % 4, k % 4

    def _block(self, b: int):
        if b not in self._cache:
            if self.ctx is None:
                self.ctx = Context()
            blocks = range(b, b + self.BLOCKS)
            ctr = np.array([[max(self.sample, 0), *self.block_of(4 * j)[:2], STREAM_TAG] for j in blocks], np.uint32)
            key = np.tile(np.array([self.seed, self.pixel], np.uint32), (len(blocks), 1))
            _, u = philox(ctr, key, self.ctx)
            for j, row in zip(blocks, u):
                self._cache[j] = row
        return self._cache[b]

    def get1D(self) -> float:
        v = float(self._block(self.dim // 4)[self.dim % 4])
        self.dim += 1
        return v

    def get2D(self):
        a = self.get1D()
        return a, self.get1D()


class GpuPathIntegrator:
    """Path integrator on the GPU wavefront: render(camera, scene, params)."""

    def __init__(self, seed: int = 0):
        self.seed = seed
        self.last_stats = None

    def render(self, camera, accel: GpuBVHAccel, params: dict, film=None, sample_offset: int = 0):
        """camera: (eye3, look3, up3, fov_deg); params: {"width", "height", "maxDepth",
        "sampleCount"}.  Returns the film (H, W, 4) float32 host array: sum of radiance
        and sample count per pixel, in the reference film's pixel order."""
        W, H = int(params["width"]), int(params["height"])
        d = self.desc(camera, W, H, int(params["sampleCount"]), int(params.get("maxDepth", 16)), sample_offset)
        if film is None:
            film = np.zeros((H, W, 4), np.float32)
        st = RenderStats()
        _check(accel.ctx.lib.spgpu_render_host(accel.ctx.h, C.byref(d), film.ctypes.data, C.byref(st)),
               "spgpu_render_host")
        self.last_stats = st
        return film

    def render_device(self, camera, accel: GpuBVHAccel, params: dict, film, sample_offset: int = 0,
                      stream: int = 0) -> RenderStats:
        """Same on a device film (torch tensor (H, W, 4) float32 on the GPU)."""
        W, H = int(params["width"]), int(params["height"])
        d = self.desc(camera, W, H, int(params["sampleCount"]), int(params.get("maxDepth", 16)), sample_offset)
        st = RenderStats()
        _check(accel.ctx.lib.spgpu_render(accel.ctx.h, C.byref(d), _ptr(film), C.byref(st),
                                          C.c_void_p(stream) if stream else None), "spgpu_render")
        self.last_stats = st
        return st

    def profile_device(self, camera, accel: GpuBVHAccel, params: dict, film, sample_offset: int = 0,
                       stream: int = 0) -> KernelProfile:
        """Per-kernel event timings and BVH visit counts of params["sampleCount"] passes."""
        W, H = int(params["width"]), int(params["height"])
        d = self.desc(camera, W, H, int(params["sampleCount"]), int(params.get("maxDepth", 16)), sample_offset)
        pr = KernelProfile()
        _check(accel.ctx.lib.spgpu_render_profile(accel.ctx.h, C.byref(d), _ptr(film), C.byref(pr),
                                                  C.c_void_p(stream) if stream else None), "spgpu_render_profile")
        return pr

    INTEGRATOR = 0   # SPGPU_INTEGRATOR_PATH

    def desc(self, camera, W, H, spp, max_depth, sample_offset=0) -> RenderDesc:
        d = RenderDesc()
        for i, v in enumerate(np.asarray(camera, np.float64).reshape(-1)[:10]):
            d.camera[i] = float(v)
        d.width, d.height, d.spp = W, H, spp
        d.sample_offset, d.max_depth, d.seed = sample_offset, max_depth, self.seed & 0xFFFFFFFF
        d.integrator = self.INTEGRATOR
        return d


class GpuDirectLightingIntegrator(GpuPathIntegrator):
    """DirectLightingIntegrator on the GPU (SPGPU_INTEGRATOR_DIRECT): emission or
    environment radiance of the camera ray plus one-light NEE at its first hit."""

    INTEGRATOR = 1


class GpuBatch:
    """Many small renders traced in one graph launch (spgpu_batch_prepare / run).
    scenes: list of scenes.Scene with width, height, spp, max_depth and camera set.
    autotune: False (0) for the streaming wavefront with its default pool, True (1) to
    time the candidates of both engines, BATCH_PERSISTENT (2) for the megakernel."""

    def __init__(self, scene_list, seed: int = 0, autotune: bool = True, device: int = 0,
                 ctx: Optional[Context] = None, pool: Optional[tuple] = None):
        self.ctx = ctx or Context(device)
        self.scenes = list(scene_list)
        self._keep = []
        items = (BatchItem * len(self.scenes))()
        integ = GpuPathIntegrator(seed=seed)
        self.offsets = []
        off = 0
        for i, sc in enumerate(self.scenes):
            v = np.ascontiguousarray(sc.verts, np.float32)
            tm = np.ascontiguousarray(sc.tri_mat, np.int32)
            m = np.ascontiguousarray(sc.materials, np.float32)
            e = None if sc.tri_emit is None else np.ascontiguousarray(sc.tri_emit, np.float32)
            self._keep += [v, tm, m, e]
            items[i].ntri = v.shape[0]
            items[i].verts = v.ctypes.data
            items[i].tri_mat = tm.ctypes.data
            items[i].nmat = m.shape[0]
            items[i].materials = m.ctypes.data
            items[i].tri_emit = e.ctypes.data if e is not None else None
            items[i].desc = integ.desc(sc.camera, sc.width, sc.height, sc.spp, sc.max_depth)
            self.offsets.append(off)
            off += sc.width * sc.height
        self.tuning = BatchTuning()
        if pool is not None:   # (slots, lanes) of the streaming pools, with autotune 0
            self.tuning.pool_slots, self.tuning.pool_lanes = int(pool[0]), int(pool[1])
        _check(self.ctx.lib.spgpu_batch_prepare(self.ctx.h, len(self.scenes), items, int(autotune),
                                                C.byref(self.tuning)), "spgpu_batch_prepare")
        self.pixels = int(self.ctx.lib.spgpu_batch_film_pixels(self.ctx.h))
        assert self.pixels == off

    def run(self, films, stream: int = 0):
        """films: device tensor of self.pixels x 4 float32 (accumulated).  Returns
        (per-render completion times in ms, RenderStats)."""
        ms = np.zeros(len(self.scenes), np.float64)
        st = RenderStats()
        _check(self.ctx.lib.spgpu_batch_run(self.ctx.h, _ptr(films), ms.ctypes.data, C.byref(st),
                                            C.c_void_p(stream) if stream else None), "spgpu_batch_run")
        return ms, st

    def profile(self, films, stream: int = 0) -> KernelProfile:
        """Per-kernel event timings of one run of a streaming batch, launched kernel by
        kernel from the host (spgpu_batch_profile); films receive two runs."""
        pr = KernelProfile()
        _check(self.ctx.lib.spgpu_batch_profile(self.ctx.h, _ptr(films), C.byref(pr),
                                                C.c_void_p(stream) if stream else None), "spgpu_batch_profile")
        return pr

    def film(self, films_host, i):
        sc = self.scenes[i]
        o = self.offsets[i]
        return films_host[o:o + sc.width * sc.height].reshape(sc.height, sc.width, 4)


class GpuGuide:
    """Learned guiding on a constructed accelerator's scene (spgpu_guiding_*)."""

    def __init__(self, accel: GpuBVHAccel, lr: float = 1e-3, bsdf_fraction: float = 0.3, batch: int = 16384,
                 seed: int = 0, capacity: int = 1 << 21, fault_injection: int = 0, guided_bounces: int = 0):
        self.accel = accel
        self.ctx = accel.ctx
        cfg = GuidingConfig(learning_rate=lr, bsdf_fraction=bsdf_fraction, batch=batch, seed=seed,
                            capacity=capacity, fault_injection=fault_injection, guided_bounces=guided_bounces)
        _check(self.ctx.lib.spgpu_guiding_init(self.ctx.h, C.byref(cfg)), "spgpu_guiding_init")

    def params(self):
        p = np.zeros(GUIDE_PARAMS, np.float32)
        _check(self.ctx.lib.spgpu_guiding_params(self.ctx.h, p.ctypes.data, 0), "spgpu_guiding_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == GUIDE_PARAMS
        _check(self.ctx.lib.spgpu_guiding_params(self.ctx.h, p.ctypes.data, 1), "spgpu_guiding_params")

    def mlp(self, features_dev, raw_dev, stream: int = 0):
        _check(self.ctx.lib.spgpu_guiding_mlp(self.ctx.h, _ptr(features_dev), features_dev.shape[0], _ptr(raw_dev),
                                              C.c_void_p(stream) if stream else None), "spgpu_guiding_mlp")

    def grad(self, samples_dev, grad_dev, stream: int = 0) -> float:
        loss = C.c_double(0.0)
        _check(self.ctx.lib.spgpu_guiding_grad(self.ctx.h, _ptr(samples_dev), samples_dev.shape[0], _ptr(grad_dev),
                                               C.byref(loss), C.c_void_p(stream) if stream else None),
               "spgpu_guiding_grad")
        return loss.value

    def render(self, camera, params: dict, film_dev, flags: int, seed: int = 0, sample_offset: int = 0,
               stream: int = 0) -> RenderStats:
        integ = GpuPathIntegrator(seed=seed)
        d = integ.desc(camera, int(params["width"]), int(params["height"]), int(params["sampleCount"]),
                       int(params.get("maxDepth", 12)), sample_offset)
        st = RenderStats()
        _check(self.ctx.lib.spgpu_guiding_render(self.ctx.h, C.byref(d), _ptr(film_dev), flags, C.byref(st),
                                                 C.c_void_p(stream) if stream else None), "spgpu_guiding_render")
        return st

    def train(self, steps: int) -> float:
        loss = C.c_double(0.0)
        _check(self.ctx.lib.spgpu_guiding_train(self.ctx.h, steps, C.byref(loss)), "spgpu_guiding_train")
        return loss.value

    def samples(self) -> int:
        return int(self.ctx.lib.spgpu_guiding_samples(self.ctx.h))

    def ring(self, max_samples: int):
        """Training ring entries (n, 16): features 9, direction 3, weight c, proposal pdf q."""
        out = np.zeros((max_samples, 16), np.float32)
        cnt = C.c_int32(0)
        _check(self.ctx.lib.spgpu_guiding_ring(self.ctx.h, out.ctypes.data, max_samples, C.byref(cnt)),
               "spgpu_guiding_ring")
        return out[:cnt.value]
