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
    for bad in (-1, 2):
        h = ctypes.c_void_p()
        rc = lib.spgpu_create(ctypes.byref(gpu.Config(device=0, wavefront=bad)), ctypes.byref(h))
        assert rc == -1 and not h.value
        assert b"wavefront" in lib.spgpu_last_error()


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
    ("spgpu_batch_profile", (None, None, None, None)),
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
    ("spgpu_bsdf_eval", (None, None, 0, None, None, None, None)),
    ("spgpu_bsdf_sample", (None, None, 0, None, None, None, None, None, None)),
    ("spgpu_sampler_generate", (None, 0, None, None, None, None)),
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


def test_header_is_plain_c_and_links(tmp_path):
    """include/spica_gpu.h compiles as strict C99 (the language of a cgo / JNI / N-API
    binding), and a C program links against the library and calls the host-only entry
    points: the version, a scene file through spgpu_scene_load, and an .hdr write."""
    import subprocess
    import pytest
    from spica_gb300 import build
    lib = build.build()
    (tmp_path / "t.ply").write_bytes(
        b"ply\nformat binary_little_endian 1.0\nelement vertex 3\nproperty float x\nproperty float y\n"
        b"property float z\nelement face 1\nproperty list uchar int vertex_indices\nend_header\n"
        + bytes.fromhex("00000000" * 3 + "0000803f" + "00000000" * 2 + "00000000" + "0000803f" + "00000000")
        + b"\x03" + bytes.fromhex("00000000" "01000000" "02000000"))
    (tmp_path / "s.xml").write_text(
        '<scene version="0.5.0"><integrator type="path"/><sensor type="perspective">'
        '<float name="fov" value="40"/><transform name="toWorld"><lookAt origin="0 0 5" target="0 0 0" up="0 1 0"/>'
        '</transform><sampler type="independent"><integer name="sampleCount" value="4"/></sampler>'
        '<film type="hdrfilm"><integer name="width" value="8"/><integer name="height" value="6"/></film></sensor>'
        '<shape type="ply"><string name="filename" value="t.ply"/></shape></scene>')
    src = tmp_path / "main.c"
    src.write_text(r'''
#include "spica_gpu.h"
#include <stdio.h>
#include <string.h>
int main(int argc, char **argv) {
    spgpu_scene_file *sf = NULL;
    uint8_t px[4 * 2 * 1] = {128, 64, 32, 129, 0, 0, 0, 0};
    if (argc < 3 || strstr(spgpu_version(), "sm_103a") == NULL) return 2;
    if (spgpu_scene_load(argv[1], &sf) != 0) { fprintf(stderr, "%s\n", spgpu_last_error()); return 3; }
    printf("%d %d %d %d %d\n", sf->ntri, sf->nmat, sf->desc.width, sf->desc.height, sf->desc.spp);
    spgpu_scene_free(sf);
    if (spgpu_scene_load("missing.xml", &sf) != SPGPU_EINVAL || sf != NULL) return 4;
    return spgpu_write_hdr(argv[2], px, 2, 1) == 0 ? 0 : 5;
}
''')
    exe = tmp_path / "main"
    inc = os.path.join(ROOT, "include")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", inc, str(src), lib,
                        "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0 and "cannot find" in r.stderr:
        pytest.skip("no C toolchain that links against the library")
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path / "s.xml"), str(tmp_path / "o.hdr")], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    assert r.stdout.split() == ["1", "1", "8", "6", "4"]
    assert (tmp_path / "o.hdr").read_bytes().startswith(b"#?RADIANCE")


def test_python_mirrors_match_the_c_structs(tmp_path):
    """Every ctypes mirror of a C-ABI struct has the C struct's size and field offsets
    (compiled with the host C compiler from include/spica_gpu.h)."""
    import ctypes
    import subprocess
    from spica_gb300 import gpu
    pairs = [("spgpu_config", gpu.Config), ("spgpu_bvh_info", gpu.BVHInfo),
             ("spgpu_trace_counters", gpu.TraceCounters), ("spgpu_render_desc", gpu.RenderDesc),
             ("spgpu_render_stats", gpu.RenderStats), ("spgpu_kernel_profile", gpu.KernelProfile),
             ("spgpu_batch_item", gpu.BatchItem), ("spgpu_batch_tuning", gpu.BatchTuning),
             ("spgpu_guiding_config", gpu.GuidingConfig), ("spgpu_scene_file", gpu.SceneFile)]
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "spica_gpu.h"', "int main(void) {"]
    for cname, py in pairs:
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, *_ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    r = subprocess.run(["gcc", "-std=c99", "-I", inc, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        parts = line.split()
        if len(parts) == 3:
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, py in pairs:
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, *_ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
