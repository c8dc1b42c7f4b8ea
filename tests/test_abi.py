"""The C-ABI library builds, loads, and exports every symbol include/*.h declares.
No compute calls: this runs without a GPU."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(spgpu_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    from spica_gb300 import build, gpu
    path = build.build()
    lib = ctypes.CDLL(path)
    declared = _declared()
    assert declared, "no declarations parsed"
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(gpu.EXPORTS) <= declared


def test_binding_declares_argument_types_for_every_export():
    """ctypes passes undeclared integer arguments as C int: a 64-bit pointer would be
    truncated, so every exported function that takes arguments declares them."""
    from spica_gb300 import gpu
    lib = gpu.load_library()
    no_args = {"spgpu_last_error", "spgpu_version"}
    undeclared = [n for n in gpu.EXPORTS if n not in no_args and getattr(lib, n).argtypes is None]
    assert not undeclared, undeclared


def test_create_rejects_invalid_pass_lanes():
    """The configuration is validated before any device call (so this runs without a
    GPU): pass_lanes outside 0..8 is refused with SPGPU_EINVAL and a message."""
    from spica_gb300 import gpu
    lib = gpu.load_library()
    for bad in (-1, 9):
        h = ctypes.c_void_p()
        rc = lib.spgpu_create(ctypes.byref(gpu.Config(device=0, pass_lanes=bad)), ctypes.byref(h))
        assert rc == -1 and not h.value
        assert b"pass_lanes" in lib.spgpu_last_error()


# every entry point with a null context or null buffers: (name, arguments)
_NULL_CALLS = [
    ("spgpu_create", (None, None)),
    ("spgpu_upload_scene", (None, 0, None, None, 0, None, None, 0, 0, None)),
    ("spgpu_build_bvh", (None,)),
    ("spgpu_bvh_stats", (None, None)),
    ("spgpu_trace", (None, 0, None, None, 0, None, None)),
    ("spgpu_trace_stats", (None, 0, None, None, 0, None, None)),
    ("spgpu_trace_host", (None, 0, None, None, 0, None)),
    ("spgpu_trace_host_noalloc", (None, 0, None, None, 0, None)),
    ("spgpu_render", (None, None, None, None, None)),
    ("spgpu_render_host", (None, None, None, None)),
    ("spgpu_render_profile", (None, None, None, None, None)),
    ("spgpu_batch_prepare", (None, 0, None, 0, None)),
    ("spgpu_batch_run", (None, None, None, None, None)),
    ("spgpu_guiding_init", (None, None)),
    ("spgpu_guiding_render", (None, None, None, 0, None, None)),
    ("spgpu_guiding_train", (None, 0, None)),
    ("spgpu_guiding_ring", (None, None, 0, None)),
    ("spgpu_guiding_params", (None, None, 0)),
    ("spgpu_guiding_mlp", (None, None, 0, None, None)),
    ("spgpu_guiding_grad", (None, None, 0, None, None, None)),
    ("spgpu_film_resolve", (None, None, 0, 0, 0, 0.0, None, None)),
    ("spgpu_write_hdr", (None, None, 0, 0)),
    ("spgpu_write_png", (None, None, 0, 0)),
    ("spgpu_scene_load", (None, None)),
    ("spgpu_load_hdr", (None, None, 0, None, None)),
]


def test_invalid_arguments_return_a_status_and_a_message():
    """Every entry point refuses a null context or null buffers with a negative status,
    before any device call (so this runs without a GPU), and leaves a message that names
    it in spgpu_last_error; spgpu_destroy and spgpu_scene_free accept NULL."""
    from spica_gb300 import gpu
    lib = gpu.load_library()
    names = {n for n, _ in _NULL_CALLS}
    counters = ("spgpu_batch_film_pixels", "spgpu_guiding_samples")   # -1 without the state they count
    assert names == {n for n in _declared() if n not in (
        "spgpu_destroy", "spgpu_scene_free", "spgpu_last_error", "spgpu_version") + counters}
    for name in counters:
        assert getattr(lib, name)(None) == -1, name
    for name, args in _NULL_CALLS:
        rc = getattr(lib, name)(*args)
        assert rc < 0, name
        assert lib.spgpu_last_error().decode().startswith(name), (name, lib.spgpu_last_error())
    lib.spgpu_destroy(None)
    lib.spgpu_scene_free(None)


def test_loader_fails_loudly_without_library(tmp_path):
    import pytest
    from spica_gb300 import gpu
    with pytest.raises(gpu.SpgpuError):
        gpu.load_library(str(tmp_path / "missing.so"))


def test_version_string():
    from spica_gb300 import gpu
    lib = gpu.load_library()
    assert b"sm_103a" in lib.spgpu_version()


def test_reference_side_plugins_compile_and_export():
    """The drop-in plugins build against the reference's own headers (only where the
    reference tree exists) and export the plugin manager's entry points."""
    import subprocess

    import pytest
    from oracle import spo
    if not os.path.isdir(spo.REF_TREE):
        pytest.skip("reference tree not present on this host")
    from spica_gb300 import build
    build.build()
    d = os.path.join(ROOT, "spica_gb300", "plugins")
    r = subprocess.run(["make", "-C", d, f"REF={spo.REF_TREE}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    for name in ("gpubvh", "gpupath", "gpudirect"):
        so = os.path.join(d, "_build", name + ".so")
        syms = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
        assert " createInstance" in syms and " getDescription" in syms, name
