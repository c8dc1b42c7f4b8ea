"""spica_gb300 -- GB300-native (sm_103a) path-tracing hot path of the spica renderer.

    from spica_gb300 import scenes, GpuBVHAccel, GpuPathIntegrator
    sc = scenes.box_room()
    accel = GpuBVHAccel(sc).construct()
    film = GpuPathIntegrator(seed=0).render(sc.camera, accel,
                                            {"width": 256, "height": 256, "maxDepth": 8, "sampleCount": 64})

The compute path is libspica_gpu.so (CUDA C++, C ABI in include/spica_gpu.h); this
package is its host-side mirror of the reference's Accelerator/Integrator plugins.
"""
from . import scenes  # noqa: F401
from .gpu import (BVHInfo, Context, GpuBatch, GpuBSDF, GpuBVHAccel, GpuDirectLightingIntegrator,  # noqa: F401
                  GpuGuide, GpuPathIntegrator, GpuSampler, RenderStats, SpgpuError, TraceCounters, load_library,
                  load_scene, philox)

__all__ = ["scenes", "Context", "GpuBatch", "GpuBSDF", "GpuSampler", "philox", "GpuBVHAccel", "GpuDirectLightingIntegrator", "GpuGuide",
           "GpuPathIntegrator", "SpgpuError", "load_library", "load_scene", "BVHInfo", "RenderStats", "TraceCounters"]
