"""Benchmark of the GPU path-tracing hot path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload: the mid-scale plain render -- 500 seeded instances of tessellated spheres
and boxes (~2.03M triangles) on a ground plane; 40% Lambert, 40% GGX conductor, 20%
dielectric; 4 quad area lights plus a 1024x512 sky with a 0.5 deg sun; 1920x1080,
max depth 16.  A step is one sample for every pixel (2,073,600 path samples) through
the wavefront integrator.  Inputs (scene, BVH, queues) are resident in HBM before the
timed region; each step's working set (~0.6 GB of queues plus ~0.12 GB of scene) is
larger than the 129 MB L2.

The JSON line carries, besides the headline path samples/s:
  e2e        the same metric through the host entry point spgpu_render_host, in render
             calls of 16 samples per pixel (the reference renders a frame's samples in
             one call): every call copies the film (float4 per pixel) host->device from
             pinned host memory, renders, and copies it back
  roofline   the closest-hit traversal kernel ("extend"), measured live: algorithmic
             bytes = rays x (32 B ray + 16 B hit + nodes/ray x 80 B + triangles/ray x
             48 B) per launch over its CUDA-event duration, against the measured HBM
             copy bandwidth
  cpu_baseline  the CPU oracle (the compiled reference where it exists, else the C++
             restatement) on a bounded sample of the same workload, all host threads
  microbench the ray-BVH intersection microbench (1,048,576-triangle displaced sphere,
             8M coherent + 8M incoherent rays), Mrays/s closest and any hit
--impl reference runs the reference's CPU implementation alone on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "path samples/s"
UNIT = "path samples/s"
CONFIG = {"workload": "mid-scale plain render: 500 instances, ~2.03M triangles, 4 area lights + 1024x512 sky, "
                      "1920x1080, max depth 16, 1 sample per pixel per step",
          "scene_seed": 0, "width": 1920, "height": 1080, "max_depth": 16,
          "l2": "per-step working set larger than L2 (no flush)", "parallelism": "replicas"}


E2E_SPP = 16   # samples per pixel per host-API render call in the end-to-end measurement
PASS_LANES = 8   # sample passes in flight (spgpu_config.pass_lanes 0 = 8)
# ncu dram__bytes_read.sum + dram__bytes_write.sum of the extend launches of the
# per-kernel profile below (one pool, 8 samples per pixel, 1920x1080), averaged per
# launch.  A constant, measured on a GB300 by
#   ncu --nvtx --nvtx-include "spgpu_render_profile/" \
#       --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum \
#       --clock-control none -k regex:k_sextend -c 120 --csv --log-file <csv> \
#       python bench.py --steps 4 --warmup 3 --no-cpu --no-micro --no-batch --no-guiding --no-e2e
# and re-measured whenever the tree, the traversal or the queue layout changes.
EXTEND_DRAM_BYTES_PER_LAUNCH = 200.47e6


def max_over_ranks(torch, x: float, ws: int, device: str = "cuda") -> float:
    """The largest of every rank's x (the job's time is its slowest replica's)."""
    if ws <= 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ws: int, units_per_rank: int, ms: float) -> float:
    """Whole-job units/s: every rank processed units_per_rank in at most ms."""
    return ws * units_per_rank / (ms / 1e3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def path_bytes(pr) -> float:
    """Algorithmic HBM bytes per path sample of the wavefront pass, from the kernels' own
    counters and this implementation's queue layout: camera ray + path state written by
    raygen (48 B) and the film count (4 B); per closest ray its traversal bytes (32 B ray,
    16 B hit, 80 B per node, 48 B per triangle), the class-queue index (4 B), the shading
    gathers (index 4 + hit 16 + ray 32 + path state 16 B) and the continuation ray and
    path state (48 B); per shadow ray its 48 B queue record written by shading and read
    back, 80 B per node and 48 B per triangle, and the film atomic (16 B)."""
    if not pr.paths:
        return 0.0
    c = pr.rays_closest / pr.paths
    sh = pr.rays_shadow / pr.paths
    closest = 32 + 16 + 80 * pr.closest_nodes_per_ray + 48 * pr.closest_tris_per_ray + 4 + 68 + 48
    shadow = 48 + 48 + 80 * pr.shadow_nodes_per_ray + 48 * pr.shadow_tris_per_ray + 16
    return 52 + c * closest + sh * shadow


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-i", str(index), "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_oracle():
    from oracle import spo
    kind = "reference" if spo.available("ref") else "port"
    if kind == "port" and not spo.available("port"):
        spo.build("port")
    return spo.Oracle("ref" if kind == "reference" else "port"), kind


def cpu_sample(scene, seconds: float = 15.0, threads: int = 0):
    """Path samples/s of the CPU oracle on a bounded sample of the workload: passes of
    1 sample per pixel over 8 film rows spread down the image (one band of 8 rows per
    step of the row index), repeated until `seconds` of work are done.
    Returns (value, kind, cores, description, build_s)."""
    o, kind = cpu_oracle()
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    sc = o.scene(scene)
    build_s = time.perf_counter() - t0
    W, H = scene.width, scene.height
    rows, bands = 8, 16
    starts = np.linspace(0, H - rows, bands).astype(int)
    total, k, t0 = 0, 0, time.perf_counter()
    while True:
        y = int(starts[k % bands])
        sc.render(scene.camera, W, H, 1, scene.max_depth, seed=9 + k // bands, window=(0, y, W, rows),
                  nthreads=threads)
        total += W * rows
        k += 1
        dt = time.perf_counter() - t0
        if dt >= seconds and k >= bands:
            break
    desc = (f"{k} bands of {rows} rows x {W} px (16 band positions spread over the image), 1 sample/pixel: "
            f"{total} path samples in {dt:.1f} s")
    return total / dt, kind, threads, desc, build_s


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from spica_gb300 import scenes
    scene = scenes.mid_scale()
    o, kind = cpu_oracle()
    threads = os.cpu_count() or 1
    sc = o.scene(scene)
    W, H = scene.width, scene.height
    rows = 8   # each step: 8 film rows (15,360 path samples), bands spread over the image
    ys = np.linspace(0, H - rows, max(args.steps, 1) + args.warmup).astype(int)
    for k in range(args.warmup):
        sc.render(scene.camera, W, H, 1, scene.max_depth, seed=100 + k, window=(0, int(ys[k]), W, rows),
                  nthreads=threads)
    t0 = time.perf_counter()
    for k in range(args.steps):
        y = int(ys[args.warmup + k])
        sc.render(scene.camera, W, H, 1, scene.max_depth, seed=200 + k, window=(0, y, W, rows), nthreads=threads)
    dt = time.perf_counter() - t0
    value = args.steps * rows * W / dt
    qbvh = None
    if kind == "reference":
        # the reference's second traversal, BVHAccel with useSIMD (its 4-wide QBVH, bvh.cc:389),
        # on the same film rows
        sq = o.scene(scene, use_simd=True)
        t0 = time.perf_counter()
        for k in range(args.steps):
            y = int(ys[args.warmup + k])
            sq.render(scene.camera, W, H, 1, scene.max_depth, seed=200 + k, window=(0, y, W, rows),
                      nthreads=threads)
        qbvh = {"value": args.steps * rows * W / (time.perf_counter() - t0), "unit": UNIT,
                "variant": "BVHAccel useSIMD=true (QBVH)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(CONFIG, step=f"{rows} film rows x {W} px, 1 sample per pixel"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{args.steps} steps of {rows} rows x {W} px", "cpu_model": cpu_model()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if qbvh:
        line["qbvh"] = qbvh
    print(json.dumps(line), flush=True)
    return 0


def cpu_trace_sample(sph, org, d, tmax, n_sample=1 << 20):
    """Closest- and any-hit Mrays/s of the CPU oracle on every host thread, on an evenly
    strided sample of the microbench's rays (coherent and incoherent halves alike)."""
    o, kind = cpu_oracle()
    t0 = time.perf_counter()
    sc = o.scene(sph)
    build_s = time.perf_counter() - t0
    idx = np.linspace(0, org.shape[0] - 1, n_sample).astype(np.int64)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    sc.trace(org[idx], d[idx], nthreads=threads)
    tc = time.perf_counter() - t0
    t0 = time.perf_counter()
    sc.trace(org[idx], d[idx], tmax[idx], any_hit=True, nthreads=threads)
    ta = time.perf_counter() - t0
    return {"closest_mrays_s": n_sample / tc / 1e6, "any_mrays_s": n_sample / ta / 1e6, "cores": threads,
            "kind": kind, "sample": f"{n_sample} of the rays (every {org.shape[0] // n_sample}th)",
            "bvh_build_s": build_s}


def microbench(torch, GpuBVHAccel, scenes, reps=3, rays=16 << 20, cpu=False):
    sph = scenes.displaced_sphere(levels=9, seed=0)
    acc = GpuBVHAccel(sph).construct()
    org, d, tmax = scenes.microbench_rays(sph, rays // 2, rays - rays // 2, 4096, 2048, seed=0)
    n = org.shape[0]
    ot = torch.zeros((n, 4), device="cuda")
    dt = torch.zeros((n, 4), device="cuda")
    ot[:, :3] = torch.from_numpy(org).cuda()
    dt[:, :3] = torch.from_numpy(d).cuda()
    dt[:, 3] = 1e32
    hits = torch.zeros((n, 4), device="cuda")
    anyo = torch.zeros(n, dtype=torch.int32, device="cuda")
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream().cuda_stream

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(reps):
            s.record()
            fn()
            e.record()
            torch.cuda.synchronize()
            best = min(best, s.elapsed_time(e))
        return best

    ms_c = timed(lambda: acc.intersect_device(ot, dt, hits, stream=stream))
    cc = acc.intersect_stats(ot, dt, hits)
    dt[:, 3] = torch.from_numpy(tmax).cuda()
    ms_a = timed(lambda: acc.intersect_device(ot, dt, anyo, any_hit=True, stream=stream))
    ca = acc.intersect_stats(ot, dt, anyo, any_hit=True)
    info = acc.info()
    out = {"triangles": int(sph.ntri), "rays": int(n), "closest_mrays_s": n / ms_c / 1e3,
           "any_mrays_s": n / ms_a / 1e3, "closest_nodes_per_ray": cc.nodes_per_ray,
           "closest_tris_per_ray": cc.tris_per_ray, "any_nodes_per_ray": ca.nodes_per_ray,
           "any_tris_per_ray": ca.tris_per_ray, "bvh_build_ms": info.build_ms, "wide_nodes": int(info.wide_nodes)}
    if cpu:
        out["cpu_baseline"] = cpu_trace_sample(sph, org, d, tmax)
    return out


def batch_bench(torch, GpuBatch, scenes, reps=3, count=64, autotune=True):
    """64 seeded box-room variants (resolution 64..512 squared, 16..256 spp) in one
    graph launch; the engine (streaming wavefront or persistent megakernel) and its
    launch shape from the autotuner."""
    vs = scenes.batch_variants(count, seed=0)
    t0 = time.perf_counter()
    b = GpuBatch(vs, seed=7, autotune=autotune)
    prep_s = time.perf_counter() - t0
    films = torch.zeros((b.pixels, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    b.run(films, stream=stream)
    torch.cuda.synchronize()
    best = None
    for _ in range(reps):
        ms, st = b.run(films, stream=stream)
        if best is None or st.ms < best[1].ms:
            best = (ms, st)
    ms, st = best
    samples = sum(v.width * v.height * v.spp for v in vs)
    return {"renders": len(vs), "path_samples": int(samples), "ms": st.ms,
            "samples_per_s": samples / (st.ms / 1e3), "mrays_s": (st.rays_closest + st.rays_shadow) / (st.ms * 1e3),
            "latency_ms_p50": float(np.percentile(ms, 50)), "latency_ms_p99": float(np.percentile(ms, 99)),
            "tuning": {"engine": {1: "streaming wavefront", 2: "persistent megakernel"}.get(b.tuning.engine),
                       "pool_slots": b.tuning.pool_slots, "pool_lanes": b.tuning.pool_lanes,
                       "iterations": b.tuning.iterations, "block": b.tuning.block,
                       "tile_pixels": b.tuning.tile_pixels, "chunk_spp": b.tuning.chunk_spp,
                       "candidates": b.tuning.candidates, "calib_ms": b.tuning.calib_ms},
            "prepare_s": prep_s}


def guiding_bench(torch, GpuBVHAccel, scenes, W=1280, H=720, budget_spp=1024, ref_spp=4096):
    """Learned guiding on the indirect-lit room (1280 x 720, max depth 12): relMSE at equal
    device time (the time of budget_spp plain samples per pixel) against the plain path
    tracer on the streaming wavefront (the default renderer; guided passes run on it too,
    collection passes pass by pass), the guided run training online for the first 25% of it
    (collection passes of 2 spp, each followed by 128 Adam steps; their samples kept in
    the image).  relMSE is taken against a ref_spp plain reference with the reference's
    own noise subtracted (its per-pixel variance from 16 independent chunks), which
    estimates the error against the converged image, as a far longer reference would.
    Also the per-sample gain of the same two images."""
    from spica_gb300 import guiding
    from spica_gb300.gpu import GpuGuide
    sc = scenes.guiding_room(width=W, height=H)
    acc = GpuBVHAccel(sc).construct()
    g = GpuGuide(acc, seed=2)
    ref, ref_var = guiding.render_reference(torch, acc, g, sc, W, H, spp=ref_spp, with_variance=True)
    noise = guiding.reference_noise(ref, ref_var)
    f = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    p = {"width": W, "height": H, "sampleCount": 8, "maxDepth": sc.max_depth}
    ms8 = min(g.render(sc.camera, p, f, 0, seed=3).ms for _ in range(3))
    budget = ms8 / 8 * budget_spp
    plain, pi = guiding.render_equal_time(torch, acc, g, sc, W, H, budget, guided=False, seed=11)
    gg = GpuGuide(acc, seed=2)
    img, gi = guiding.render_equal_time(torch, acc, gg, sc, W, H, budget, guided=True, seed=11, train_steps=128,
                                        keep_training_samples=1.0)
    raw_p, raw_g = guiding.relmse(plain, ref), guiding.relmse(img, ref)
    e_p, e_g = raw_p - noise, raw_g - noise   # against the converged image
    # training kernel throughput: 64 Adam steps on the trained ring, CUDA events
    steps = 64
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    gg.train(steps)
    ev1.record()
    torch.cuda.synchronize()
    step_ms = ev0.elapsed_time(ev1) / steps
    flop = 16384 * (22656 + 45312)   # batch x (forward + backward) per step; Adam is O(params)
    peak, src = bf16_peak()
    train_roof = {"bound": "tensor", "achieved": flop / (step_ms / 1e3) / 1e12, "peak": peak, "unit": "TFLOP/s",
                  "frac": flop / (step_ms / 1e3) / 1e12 / peak, "peak_source": src, "ms_per_step": step_ms,
                  "flop_per_step": flop}
    return {"scene": "indirect-lit room, 2418 tris", "width": W, "height": H, "reference_spp": ref_spp,
            "wavefront": "streaming (plain and guided passes), pass by pass (collection passes)",
            "budget_ms": budget, "relmse_plain": e_p, "relmse_guided": e_g, "equal_time_gain": e_p / e_g,
            "relmse_reference_noise": noise, "equal_time_gain_raw": raw_p / raw_g,
            "per_sample_gain": (e_p * pi["render_spp"] / (e_g * (gi["render_spp"] + gi["kept_training_spp"]))
                                if gi["render_spp"] else None),
            "plain_spp": pi["render_spp"], "guided_spp": gi["render_spp"] + gi["kept_training_spp"],
            "adam_steps": gi["adam_steps"],
            "training_spp": gi["training_spp"], "train_fraction": 0.25,
            "plain_ms_per_spp": ms8 / 8,
            "guided_ms_per_spp": gi["render_ms"] / max(gi["render_spp"], 1),
            "collect_ms_per_spp": gi["collect_ms"] / max(gi["training_spp"], 1),
            "train_ms_per_step": gi["train_ms"] / max(gi["adam_steps"], 1),
            "training_roofline": train_roof}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-micro", action="store_true", help="skip the intersection microbench")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-renders measurement")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end host-API measurement")
    ap.add_argument("--no-guiding", action="store_true", help="skip the learned-guiding comparison")
    ap.add_argument("--no-profile", action="store_true", help="skip the per-kernel profile (roofline)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from spica_gb300 import GpuBatch, GpuBVHAccel, GpuPathIntegrator, scenes
    from spica_gb300.gpu import KERNEL_CLASSES

    scene = scenes.mid_scale()
    W, H, md = scene.width, scene.height, scene.max_depth
    npix = W * H
    acc = GpuBVHAccel(scene, device=local).construct()
    info = acc.info()
    integ = GpuPathIntegrator(seed=1234 + rank)
    params = {"width": W, "height": H, "maxDepth": md}
    film = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # warm-up: every pass lane allocates its queues and captures its graph on its first
    # pass, so the warm-up renders W passes on each of the PASS_LANES lanes
    warm = max(args.warmup, 1) * PASS_LANES
    integ.render_device(scene.camera, acc, dict(params, sampleCount=warm), film, stream=stream)
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    st = integ.render_device(scene.camera, acc, dict(params, sampleCount=args.steps), film,
                             sample_offset=warm, stream=stream)
    ev1.record()
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(torch, ev0.elapsed_time(ev1), ws, device="cuda")
    value = replica_throughput(ws, args.steps * npix, ms)
    rays = st.rays_closest + st.rays_shadow

    # end to end through the host entry point: render calls of E2E_SPP samples per pixel
    # (the reference renders all of a frame's samples in one call), each copying the
    # pinned host film to the device and back
    film_bytes = npix * 16
    e2e_value = None
    e2e_calls = max(1, (args.steps + E2E_SPP - 1) // E2E_SPP)
    if not args.no_e2e:
        host_film = torch.zeros((H, W, 4), dtype=torch.float32).pin_memory()
        hf = host_film.numpy()
        integ.render(scene.camera, acc, dict(params, sampleCount=E2E_SPP), film=hf, sample_offset=1 << 16)
        barrier()
        t0 = time.perf_counter()
        for k in range(e2e_calls):
            integ.render(scene.camera, acc, dict(params, sampleCount=E2E_SPP), film=hf,
                         sample_offset=(1 << 16) + E2E_SPP * (k + 1))
        barrier()
        e2e_s = time.perf_counter() - t0
        e2e_value = ws * e2e_calls * E2E_SPP * npix / e2e_s

    if rank != 0:
        return 0

    if args.no_profile:
        print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                          "config": dict(CONFIG, width=W, height=H), "profiling_case": True}), flush=True)
        return 0
    # per-kernel profile: the same render kernel by kernel, each launch event-timed, then
    # again with visit counters (8 samples per pixel: the pool refills 8 times)
    prof_film = torch.zeros_like(film)
    pr = integ.profile_device(scene.camera, acc, dict(params, sampleCount=8), prof_film, sample_offset=1 << 20,
                              stream=stream)
    total_k = sum(pr.kernel_ms[i] for i in range(7))
    kernels = {KERNEL_CLASSES[i]: {"ms": pr.kernel_ms[i], "launches": int(pr.launches[i]),
                                   "share": pr.kernel_ms[i] / total_k if total_k else 0.0} for i in range(7)}
    ext_ms_per_launch = pr.kernel_ms[1] / max(pr.launches[1], 1)
    rays_per_launch = pr.rays_closest / max(pr.launches[1], 1)
    bytes_per_ray = 32 + 16 + 80 * pr.closest_nodes_per_ray + 48 * pr.closest_tris_per_ray
    hbm, peak_src = peaks()
    achieved = rays_per_launch * bytes_per_ray / (ext_ms_per_launch / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "extend (closest-hit traversal)", "achieved": achieved, "peak": hbm,
                "unit": "GB/s", "frac": achieved / hbm, "peak_source": peak_src,
                "traffic": None, "bytes_per_ray": bytes_per_ray, "rays_per_launch": rays_per_launch,
                "ms_per_launch": ext_ms_per_launch, "nodes_per_ray": pr.closest_nodes_per_ray,
                "tris_per_ray": pr.closest_tris_per_ray}
    if (W, H) == (1920, 1080):
        roofline["traffic"] = EXTEND_DRAM_BYTES_PER_LAUNCH

    pb = path_bytes(pr)
    path_roof = {"bound": "hbm", "bytes_per_path": pb, "achieved": value / ws * pb / 1e9, "peak": hbm, "unit": "GB/s",
                 "frac": value / ws * pb / 1e9 / hbm}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": dict(CONFIG, triangles=int(scene.ntri), wide_nodes=int(info.wide_nodes),
                           bvh_build_ms=info.build_ms),
            "mrays_s": ws * args.steps * rays / max(st.paths, 1) * npix / (ms / 1e3) / 1e6 if st.paths else None,
            "rays_per_path": rays / max(st.paths, 1),
            "e2e": None if e2e_value is None else {"value": e2e_value, "unit": UNIT,
                                                   "h2d_bytes_per_step": (film_bytes + 80) / E2E_SPP,
                                                   "d2h_bytes_per_step": film_bytes / E2E_SPP,
                                                   "samples_per_call": E2E_SPP, "calls": e2e_calls},
            "gpu_launches": int(st.kernel_launches), "clocks": clk, "roofline": roofline,
            "path_roofline": path_roof,
            "kernels": kernels}
    if not args.no_micro:
        line["microbench"] = microbench(torch, GpuBVHAccel, scenes, cpu=not args.no_cpu and ws == 1)
    if not args.no_batch:
        line["batch"] = batch_bench(torch, GpuBatch, scenes)
    if not args.no_guiding:
        line["guiding"] = guiding_bench(torch, GpuBVHAccel, scenes)
    if not args.no_cpu and ws == 1:
        v, kind, cores, desc, build_s = cpu_sample(scene)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": desc,
                                "bvh_build_s": build_s, "cpu_model": cpu_model()}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
