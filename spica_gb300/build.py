"""Build libspica_gpu.so (the C-ABI library) for sm_103a with nvcc, in-tree.

    python -m spica_gb300.build          # or spica_gb300.build.build()

Each CUDA translation unit is compiled in parallel, then linked into
spica_gb300/_build/libspica_gpu.so against the static CUDA runtime.  No torch
types cross the boundary, so the library loads without torch.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libspica_gpu.so")
SOURCES = ["api.cu", "bvh.cu", "wavefront.cu", "stream.cu", "batch.cu", "guide.cu", "film.cu", "bsdf.cu", "sceneio.cc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unknown-pragmas",
         "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout[-6000:] + r.stderr[-6000:])
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "spica_gpu.h"))
    nv = nvcc()
    flags = FLAGS + list(extra_flags or [])
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        if _stale(o, [s] + headers + [__file__]):
            jobs.append([nv, *ARCH, *flags, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    objs = [os.path.join(OUT, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    if _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-o", LIB, *objs])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
