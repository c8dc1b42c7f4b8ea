"""Equal-time comparison of guided and plain rendering (the learned-guiding workload).

relmse(I, R) = mean over pixels and channels of (I - R)^2 / (R^2 + 1e-2), against a
high-sample plain reference R.  render_equal_time() spends the same device time on
either method: the guided run trains online for the first `train_fraction` of it
(collection passes + Adam steps), then renders with the trained proposal; only the
samples of the rendering phase enter its image.
"""
from __future__ import annotations

import time

import numpy as np

from .gpu import GUIDE_COLLECT, GUIDE_GUIDED, GpuBVHAccel, GpuGuide


def relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def _mean(film):
    f = film.detach().cpu().numpy() if hasattr(film, "detach") else film
    return f[..., :3] / np.maximum(f[..., 3:4], 1)


def reference_noise(ref, ref_var):
    """The reference's own share of relmse(img, ref): E[(I - R)^2] = E[(I - mu)^2] +
    Var(R) for an image I independent of the reference R, so subtracting this term
    from relmse gives the error against the converged image."""
    return float(np.mean(ref_var / (ref ** 2 + 1e-2)))


def render_reference(torch, accel: GpuBVHAccel, guide: GpuGuide, scene, W, H, spp, seed=777, chunk=256,
                     with_variance=False):
    """Plain high-sample reference (same estimator, plain BSDF sampling); with
    with_variance, also the per-pixel variance of its mean, from the spread of the
    chunk means (spp // chunk independent chunks)."""
    film = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    s1 = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
    s2 = torch.zeros_like(s1)
    prev = film[..., :3].double().clone()
    done, chunks = 0, 0
    while done < spp:
        n = min(chunk, spp - done)
        guide.render(scene.camera, {"width": W, "height": H, "sampleCount": n, "maxDepth": scene.max_depth}, film, 0,
                     seed=seed, sample_offset=done)
        done += n
        if with_variance:
            cur = film[..., :3].double()
            m = (cur - prev) / n
            s1 += m
            s2 += m * m
            prev = cur.clone()
            chunks += 1
    torch.cuda.synchronize()
    if not with_variance:
        return _mean(film)
    mean_c = s1 / chunks
    var = ((s2 / chunks - mean_c * mean_c) * chunks / max(chunks - 1, 1) / chunks).clamp_min(0.0)
    return _mean(film), var.cpu().numpy()


def render_equal_time(torch, accel: GpuBVHAccel, guide: GpuGuide, scene, W, H, budget_ms, guided: bool,
                      train_fraction=0.25, train_steps=16, collect_spp=2, chunk_spp=8, seed=1,
                      keep_training_samples=0.0):
    """Render for budget_ms of device time (training included for the guided run);
    returns (mean image, info).  Launches carry chunk_spp samples per pixel.

    The guided run's collection passes are unbiased renders too: with
    keep_training_samples = f > 0, the samples of the last fraction f of the training
    passes (by time) are kept in the image, the earlier ones (from a barely trained
    network) only feed the training ring."""
    p = {"width": W, "height": H, "maxDepth": scene.max_depth}
    film = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    spent, spp, trained, offset, losses, kept = 0.0, 0, 0, 0, [], 0
    collect_ms = train_ms = render_ms = 0.0
    if guided:
        scratch = torch.zeros_like(film)
        t_train = train_fraction * budget_ms
        while spent < t_train:
            keep = keep_training_samples > 0 and spent >= (1.0 - keep_training_samples) * t_train
            st = guide.render(scene.camera, dict(p, sampleCount=collect_spp), film if keep else scratch,
                              GUIDE_GUIDED | GUIDE_COLLECT, seed=seed + 1000, sample_offset=offset)
            offset += collect_spp
            kept += collect_spp if keep else 0
            t0 = time.perf_counter()
            losses.append(guide.train(train_steps))
            torch.cuda.synchronize()
            dt = 1e3 * (time.perf_counter() - t0)
            spent += st.ms + dt
            collect_ms += st.ms
            train_ms += dt
            trained += train_steps
    flags = GUIDE_GUIDED if guided else 0
    while spent < budget_ms:
        st = guide.render(scene.camera, dict(p, sampleCount=chunk_spp), film, flags, seed=seed, sample_offset=spp)
        spent += st.ms
        render_ms += st.ms
        spp += chunk_spp
    torch.cuda.synchronize()
    return _mean(film), {"ms": spent, "render_spp": spp, "adam_steps": trained, "training_spp": offset,
                         "kept_training_spp": kept, "collect_ms": collect_ms, "train_ms": train_ms,
                         "render_ms": render_ms,
                         "loss_first": losses[0] if losses else None, "loss_last": losses[-1] if losses else None}
