"""spgpu_trace_host_noalloc (host ray buffers, static device scratch, no device
allocation) against spgpu_trace_host on the same rays: two calls in a row must return
exactly what the allocating entry point returns, both in this process (after whatever
tests ran before; this file is collected last) and in a fresh process whose first
call does the scratch set-up."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

pytestmark = pytest.mark.gpu

MAX_RAYS = 65536


def _rays(n, seed):
    """Rays from a shell around the unit sphere toward random points near it: hits,
    grazing rays and misses."""
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(n, 3))
    o *= (2.0 + rng.random((n, 1))) / np.linalg.norm(o, axis=1, keepdims=True)
    target = rng.normal(size=(n, 3)) * 0.9
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmax = rng.uniform(0.5, 4.0, n)
    return o.astype(np.float32), d.astype(np.float32), tmax.astype(np.float32)


def check_two_calls():
    from spica_gb300 import GpuBVHAccel, scenes
    from spica_gb300.gpu import SpgpuError
    acc = GpuBVHAccel(scenes.displaced_sphere(levels=5)).construct()
    o, d, tmax = _rays(MAX_RAYS - 123, seed=5)
    prim, t, u, v = acc.intersect(o, d)
    occluded = acc.intersect_any(o, d, tmax)
    assert (prim >= 0).any() and (prim < 0).any()
    for _ in range(2):
        p2, t2, u2, v2 = acc.intersect_noalloc(o, d)
        np.testing.assert_array_equal(p2, prim)
        np.testing.assert_array_equal(t2, t)
        np.testing.assert_array_equal(u2, u)
        np.testing.assert_array_equal(v2, v)
        np.testing.assert_array_equal(acc.intersect_noalloc(o, d, tmax, any_hit=True), occluded)
    # a batch above the static limit is refused with a clear error
    ob, db, _ = _rays(MAX_RAYS + 1, seed=6)
    with pytest.raises(SpgpuError, match="static scratch limit"):
        acc.intersect_noalloc(ob, db)
    # an exactly full batch still works
    of, df, _ = _rays(MAX_RAYS, seed=7)
    np.testing.assert_array_equal(acc.intersect_noalloc(of, df)[0], acc.intersect(of, df)[0])


def test_noalloc_trace_matches_allocating_trace(gpulib):
    check_two_calls()


def test_noalloc_trace_in_fresh_process(gpulib):
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, os.path.abspath(__file__)], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "noalloc ok" in r.stdout


if __name__ == "__main__":
    check_two_calls()
    print("noalloc ok")
