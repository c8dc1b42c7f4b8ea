"""Small, fixed workloads for kernel profiling (ncu captures of one kernel on a small
case), separate from the benchmark:

    python -m spica_gb300.profcases render [--width W] [--height H] [--spp N] [--warmup K]
    python -m spica_gb300.profcases micro [--rays N]
    python -m spica_gb300.profcases batch [--renders N] [--engine stream|persistent] [--no-graph]
    python -m spica_gb300.profcases guided [--wavefront 0|1]
    python -m spica_gb300.profcases train
    python -m spica_gb300.profcases build [--levels L]
    python -m spica_gb300.profcases film [--width W] [--height H]

render  the mid-scale scene (500 instances, ~2.03M triangles, depth 16) at W x H:
        a warm-up render of 8 K samples per pixel, then a render of N samples per pixel
        inside the NVTX range "profiled" (streaming wavefront: k_sregen, k_sextend,
        k_sshade<0..2>, k_sshadow, k_sadvance)
micro   the intersection microbench's sphere (1,048,576 triangles) and N of its rays,
        closest then any hit (k_trace)
batch   the first N seeded box-room variants as one batch: with --engine stream (the
        default) its graph run, then the same batch kernel by kernel from the host inside
        the NVTX range "profiled" (k_sregen, k_sextend, k_sshade<0..2>, k_sshadow,
        k_sadvance, their batch forms; --no-graph skips the graph run); with --engine
        persistent the megakernel (k_batch)
guided  the guiding room at 640 x 360: 8 collection passes of 2 spp with 32 Adam steps
        each (k_collect, k_gather, k_guide_train, k_grad_sum), then one plain and one guided
        render of 8 spp inside the NVTX range "profiled" (k_sshade_guided on the streaming
        wavefront; k_shade_guided with --wavefront 1, pass by pass), then one network
        evaluation of 65,536 inputs (k_guide_forward)
train   the guiding room at 1280 x 720: 8 collection passes of 2 spp, 16 + 64 Adam steps
        of 16,384 samples (host-timed), then 20 steps inside the NVTX range "profiled"
        (k_gather, k_guide_train, k_grad_sum, k_guide_pack)
build   the device BVH build of the mid-scale scene, or of the microbench sphere with
        --levels (Morton keys, clustering rounds, SAH programme, collapse)
film    a rendered box room at W x H resolved by every film format (RGBE, gamma,
        Reinhard, Drago, Durand)
Each prints one JSON line of its own timings.
"""
from __future__ import annotations

import argparse
import json
import sys


def _render(args, torch):
    from . import GpuBVHAccel, GpuPathIntegrator, scenes
    sc = scenes.mid_scale(width=args.width, height=args.height)
    acc = GpuBVHAccel(sc).construct()
    integ = GpuPathIntegrator(seed=1234)
    p = {"width": sc.width, "height": sc.height, "maxDepth": sc.max_depth}
    film = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
    integ.render_device(sc.camera, acc, dict(p, sampleCount=8 * max(args.warmup, 1)), film)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("profiled")
    st = integ.render_device(sc.camera, acc, dict(p, sampleCount=args.spp), film, sample_offset=1 << 12)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    return {"case": "render", "width": sc.width, "height": sc.height, "spp": args.spp, "ms": st.ms,
            "paths": int(st.paths)}


def _micro(args, torch):
    from . import GpuBVHAccel, scenes
    sph = scenes.displaced_sphere(levels=9, seed=0)
    acc = GpuBVHAccel(sph).construct()
    org, d, tmax = scenes.microbench_rays(sph, args.rays // 2, args.rays - args.rays // 2, 4096, 2048, seed=0)
    n = org.shape[0]
    ot = torch.zeros((n, 4), device="cuda")
    dt = torch.zeros((n, 4), device="cuda")
    ot[:, :3] = torch.from_numpy(org).cuda()
    dt[:, :3] = torch.from_numpy(d).cuda()
    dt[:, 3] = 1e32
    hits = torch.zeros((n, 4), device="cuda")
    anyo = torch.zeros(n, dtype=torch.int32, device="cuda")
    acc.intersect_device(ot, dt, hits)
    acc.intersect_device(ot, dt, hits)
    dt[:, 3] = torch.from_numpy(tmax).cuda()
    acc.intersect_device(ot, dt, anyo, any_hit=True)
    torch.cuda.synchronize()
    return {"case": "micro", "rays": n}


def _batch(args, torch):
    from . import GpuBatch, scenes
    from .gpu import BATCH_PERSISTENT, KERNEL_CLASSES
    vs = scenes.batch_variants(64, seed=0)[:args.renders]
    persistent = args.engine == "persistent"
    b = GpuBatch(vs, seed=7, autotune=BATCH_PERSISTENT if persistent else 0)
    films = torch.zeros((b.pixels, 4), dtype=torch.float32, device="cuda")
    out = {"case": "batch", "engine": args.engine, "renders": len(vs)}
    if not args.no_graph:
        b.run(films)
        ms, st = b.run(films)
        torch.cuda.synchronize()
        out.update(ms=st.ms, samples_per_s=st.paths / (st.ms / 1e3))
    if not persistent:
        # the same batch kernel by kernel from the host, inside the NVTX range "profiled"
        torch.cuda.nvtx.range_push("profiled")
        pr = b.profile(films)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out["kernel_ms"] = {n: pr.kernel_ms[k] for k, n in enumerate(KERNEL_CLASSES)}
        out["launches"] = {n: pr.launches[k] for k, n in enumerate(KERNEL_CLASSES)}
    return out


def _guided(args, torch):
    import numpy as np

    from . import Context, GpuBVHAccel, scenes
    from .gpu import GUIDE_COLLECT, GUIDE_GUIDED, GpuGuide
    W, H = 640, 360
    sc = scenes.guiding_room(width=W, height=H)
    acc = GpuBVHAccel(sc, ctx=Context(0, wavefront=args.wavefront)).construct()
    g = GpuGuide(acc, seed=2)
    p = {"width": W, "height": H, "maxDepth": sc.max_depth}
    f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    for k in range(8):
        g.render(sc.camera, dict(p, sampleCount=2), f, GUIDE_GUIDED | GUIDE_COLLECT, seed=1, sample_offset=2 * k)
        g.train(32)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("profiled")
    sp = g.render(sc.camera, dict(p, sampleCount=8), f, 0, seed=2)
    sg = g.render(sc.camera, dict(p, sampleCount=8), f, GUIDE_GUIDED, seed=2)
    torch.cuda.nvtx.range_pop()
    feats = torch.from_numpy(np.random.default_rng(3).random((65536, 9)).astype(np.float32)).cuda()
    raw = torch.zeros((65536, 40), dtype=torch.float32, device="cuda")
    g.mlp(feats, raw)
    torch.cuda.synchronize()
    return {"case": "guided", "width": W, "height": H, "spp": 8, "wavefront": args.wavefront, "plain_ms": sp.ms,
            "guided_ms": sg.ms}


def _train(args, torch):
    import time

    from . import GpuBVHAccel, scenes
    from .gpu import GUIDE_COLLECT, GUIDE_GUIDED, GpuGuide
    W, H = 1280, 720
    sc = scenes.guiding_room(width=W, height=H)
    acc = GpuBVHAccel(sc).construct()
    g = GpuGuide(acc, seed=2)
    p = {"width": W, "height": H, "maxDepth": sc.max_depth}
    f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    for k in range(8):
        g.render(sc.camera, dict(p, sampleCount=2), f, GUIDE_GUIDED | GUIDE_COLLECT, seed=1, sample_offset=2 * k)
    g.train(16)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.train(64)
    torch.cuda.synchronize()
    step_ms = (time.perf_counter() - t0) * 1e3 / 64
    torch.cuda.nvtx.range_push("profiled")
    g.train(20)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    return {"case": "train", "width": W, "height": H, "ring": int(g.samples()), "batch": 16384,
            "ms_per_step_host": step_ms}


def _build(args, torch):
    from . import GpuBVHAccel, scenes
    sc = scenes.displaced_sphere(levels=args.levels, seed=0) if args.levels else scenes.mid_scale()
    acc = GpuBVHAccel(sc).construct()
    acc.construct()
    info = acc.info()
    return {"case": "build", "triangles": int(info.triangles), "wide_nodes": int(info.wide_nodes),
            "build_ms": info.build_ms}


def _film(args, torch):
    from . import GpuBVHAccel, GpuPathIntegrator, scenes
    from .gpu import FILM_DRAGO, FILM_DURAND, FILM_GAMMA_BYTES, FILM_REINHARD, FILM_RGBE, film_resolve
    sc = scenes.box_room(width=args.width, height=args.height)
    acc = GpuBVHAccel(sc).construct()
    film = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda")
    GpuPathIntegrator(seed=1).render_device(sc.camera, acc, {"width": sc.width, "height": sc.height, "maxDepth": 8,
                                                             "sampleCount": 16}, film)
    formats = [(FILM_RGBE, 0.0), (FILM_GAMMA_BYTES, 2.2), (FILM_REINHARD, 0.18), (FILM_DRAGO, 0.85),
               (FILM_DURAND, 5.0)]
    for fmt, param in formats:
        film_resolve(acc.ctx, film, fmt, param)
    torch.cuda.synchronize()
    return {"case": "film", "width": sc.width, "height": sc.height, "formats": [f for f, _ in formats]}


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m spica_gb300.profcases")
    ap.add_argument("case", choices=["render", "micro", "batch", "guided", "train", "build", "film"])
    ap.add_argument("--width", type=int, default=960)
    ap.add_argument("--height", type=int, default=540)
    ap.add_argument("--spp", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--rays", type=int, default=1 << 21)
    ap.add_argument("--renders", type=int, default=4)
    ap.add_argument("--levels", type=int, default=0)
    ap.add_argument("--wavefront", type=int, default=0, choices=[0, 1])
    ap.add_argument("--engine", default="stream", choices=["stream", "persistent"])
    ap.add_argument("--no-graph", action="store_true", help="batch: skip the graph runs, profile only")
    args = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(0)
    fn = {"render": _render, "micro": _micro, "batch": _batch, "guided": _guided, "train": _train, "build": _build,
          "film": _film}
    print(json.dumps(fn[args.case](args, torch)), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
