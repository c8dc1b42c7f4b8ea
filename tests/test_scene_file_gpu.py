"""A scene file rendered on the GPU: the box room written in the reference's XML format
(PLY meshes, diffuse BSDFs, an area emitter) and loaded by spgpu_scene_load renders
the film of the procedurally built box room with the same camera: the same samples,
equal up to the order in which concurrent pass lanes add into the film (last bits)."""
import numpy as np
import pytest

from spica_gb300 import GpuBVHAccel, GpuPathIntegrator, scenes
from spica_gb300.gpu import load_scene
from test_scene_file import scene_to_files

pytestmark = pytest.mark.gpu


def test_scene_file_renders_like_the_procedural_scene(gpulib, tmp_path):
    sc = scenes.box_room(width=48, height=32, spp=8, max_depth=6)
    got, integ = load_scene(scene_to_files(sc, tmp_path / "box"))
    assert integ == "path"
    p = {"width": got.width, "height": got.height, "maxDepth": got.max_depth, "sampleCount": got.spp}
    f_file = GpuPathIntegrator(seed=3).render(got.camera, GpuBVHAccel(got).construct(), p)
    f_proc = GpuPathIntegrator(seed=3).render(got.camera, GpuBVHAccel(sc).construct(), p)
    assert np.all(f_file[..., 3] == got.spp) and f_file[..., :3].sum() > 0
    np.testing.assert_array_equal(f_file[..., 3], f_proc[..., 3])
    np.testing.assert_allclose(f_file[..., :3], f_proc[..., :3], rtol=1e-5, atol=1e-6)
