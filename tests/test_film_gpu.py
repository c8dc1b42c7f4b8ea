"""Film output on the device (spgpu_film_resolve) against the compiled reference's
outputs for the same float film (tests/golden/film_output.npz): the .hdr file byte for
byte, LDRFilm's gamma-2.2 bytes, the images of ReinhardTmo, DragoTmo and DurandTMO."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_film import parse_hdr

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_rgbe_resolve_and_file_match_reference(gpulib, tmp_path):
    from spica_gb300 import gpu
    g = np.load(os.path.join(GOLDEN, "film_output.npz"))
    ctx = gpu.Context(0)
    rgbe = gpu.film_resolve(ctx, _dev(g["film"]), gpu.FILM_RGBE).cpu().numpy()
    _, _, ref_px = parse_hdr(bytes(g["hdr"]))
    np.testing.assert_array_equal(rgbe, ref_px)
    path = tmp_path / "film.hdr"
    gpu.write_hdr(str(path), rgbe)
    assert path.read_bytes() == bytes(g["hdr"])


def test_gamma_bytes_match_reference(gpulib):
    from spica_gb300 import gpu
    g = np.load(os.path.join(GOLDEN, "film_output.npz"))
    ctx = gpu.Context(0)
    out = gpu.film_resolve(ctx, _dev(g["film"]), gpu.FILM_GAMMA_BYTES, 2.2).cpu().numpy()
    diff = np.abs(out.astype(int) - g["gamma22"].astype(int))
    # FP64 pow on the device and in the host libm may differ in the last ulp: a byte can
    # flip only where 255 * v lies within an ulp of an integer
    assert diff.max() <= 1 and (diff > 0).mean() < 1e-3, (diff.max(), (diff > 0).mean())


def test_reinhard_matches_reference(gpulib):
    from spica_gb300 import gpu
    g = np.load(os.path.join(GOLDEN, "film_output.npz"))
    ctx = gpu.Context(0)
    out = gpu.film_resolve(ctx, _dev(g["film"]), gpu.FILM_REINHARD, 0.18).cpu().numpy()
    # float output of FP64 arithmetic; the log-mean is summed in a different order
    np.testing.assert_allclose(out, g["reinhard"], rtol=2e-6, atol=1e-30)


def test_drago_matches_reference(gpulib):
    from spica_gb300 import gpu
    g = np.load(os.path.join(GOLDEN, "film_output.npz"))
    ctx = gpu.Context(0)
    out = gpu.film_resolve(ctx, _dev(g["film"]), gpu.FILM_DRAGO, 0.85).cpu().numpy()
    # float output of FP64 arithmetic; the log-mean is summed in a different order
    np.testing.assert_allclose(out, g["drago"], rtol=2e-6, atol=1e-30)


def test_durand_matches_reference(gpulib):
    from spica_gb300 import gpu
    g = np.load(os.path.join(GOLDEN, "film_output.npz"))
    ctx = gpu.Context(0)
    out = gpu.film_resolve(ctx, _dev(g["film"]), gpu.FILM_DURAND, 5.0).cpu().numpy()
    # float output of FP64 arithmetic (device pow / log10 may differ from the host libm in
    # the last ulp), clamped to [0, 1] as the reference clamps
    np.testing.assert_allclose(out, g["durand"], rtol=2e-6, atol=1e-12)


def test_durand_on_a_rendered_film_matches_restatement(gpulib):
    """A larger film (a box-room render, 320 x 200) through the device Durand operator
    against the numpy restatement of the reference's operator."""
    import torch
    from oracle import tmo_oracle
    from spica_gb300 import GpuBVHAccel, GpuPathIntegrator, gpu, scenes
    sc = scenes.box_room(width=320, height=200)
    acc = GpuBVHAccel(sc).construct()
    film = torch.zeros((200, 320, 4), dtype=torch.float32, device="cuda")
    GpuPathIntegrator(seed=3).render_device(sc.camera, acc, {"width": 320, "height": 200, "maxDepth": 6,
                                                              "sampleCount": 4}, film)
    out = gpu.film_resolve(acc.ctx, film, gpu.FILM_DURAND, 8.0).cpu().numpy()
    ref = tmo_oracle.durand(film.cpu().numpy(), 8.0)
    np.testing.assert_allclose(out, ref, rtol=2e-6, atol=1e-12)
    dr = gpu.film_resolve(acc.ctx, film, gpu.FILM_DRAGO, 0.7).cpu().numpy()
    np.testing.assert_allclose(dr, tmo_oracle.drago(film.cpu().numpy(), 0.7), rtol=2e-6, atol=1e-30)


def test_rendered_film_to_files(gpulib, tmp_path):
    """The render -> resolve -> write path end to end on a box-room film."""
    import torch
    from spica_gb300 import GpuBVHAccel, GpuPathIntegrator, gpu, scenes
    sc = scenes.box_room(width=64, height=48)
    acc = GpuBVHAccel(sc).construct()
    film = torch.zeros((48, 64, 4), dtype=torch.float32, device="cuda")
    GpuPathIntegrator(seed=1).render_device(sc.camera, acc, {"width": 64, "height": 48, "maxDepth": 8,
                                                              "sampleCount": 16}, film)
    rgbe = gpu.film_resolve(acc.ctx, film, gpu.FILM_RGBE).cpu().numpy()
    gpu.write_hdr(str(tmp_path / "box.hdr"), rgbe)
    W, H, px = parse_hdr((tmp_path / "box.hdr").read_bytes())
    assert (W, H) == (64, 48) and np.array_equal(px, rgbe) and rgbe[..., 3].max() > 0
    ldr = gpu.film_resolve(acc.ctx, film, gpu.FILM_GAMMA_BYTES, 2.2).cpu().numpy()
    gpu.write_png(str(tmp_path / "box.png"), ldr)
    assert ldr.max() > 0
