"""Scene files of the reference's XML format through spgpu_scene_load (CPU): the PLY
loader, the transform elements and the .hdr reader against the compiled reference's
own meshio::loadPLY, Transform and Image::loadHdr (bit for bit, where the reference
tree exists); the box room written as a scene file reads back as the arrays the
procedural builder makes; the parameter store's persistence and consumption rules;
OBJ meshes; and refusals of what the GPU path does not render."""
import os
import struct

import numpy as np
import pytest

from spica_gb300 import scenes
from spica_gb300.gpu import SpgpuError, load_hdr, load_scene, write_hdr


def write_ply(path, verts, faces):
    """Binary little-endian PLY with float x, y, z and uchar-int face lists."""
    verts = np.asarray(verts, np.float32).reshape(-1, 3)
    with open(path, "wb") as f:
        f.write(b"ply\nformat binary_little_endian 1.0\ncomment written by the scene-file tests\n")
        f.write(f"element vertex {len(verts)}\nproperty float x\nproperty float y\nproperty float z\n".encode())
        f.write(f"element face {len(faces)}\nproperty list uchar int vertex_indices\nend_header\n".encode())
        f.write(verts.astype("<f4").tobytes())
        for face in faces:
            f.write(struct.pack("<B", len(face)) + np.asarray(face, "<i4").tobytes())


def rgb(v):
    return " ".join(repr(float(x)) for x in v)


def bsdf_xml(m, ident):
    t = int(m[0])
    if t == scenes.MAT_LAMBERT:
        return f'<bsdf type="diffuse" id="{ident}"><rgb name="reflectance" value="{rgb(m[1:4])}"/></bsdf>'
    if t == scenes.MAT_DIELECTRIC:
        return (f'<bsdf type="dielectric" id="{ident}"><rgb name="specularReflectance" value="1 1 1"/>'
                f'<rgb name="specularTransmittance" value="1 1 1"/><float name="intIOR" value="{float(m[1])!r}"/></bsdf>')
    if t == scenes.MAT_PLASTIC:
        return (f'<bsdf type="plastic" id="{ident}"><rgb name="diffuseReflectance" value="{rgb(m[1:4])}"/>'
                f'<rgb name="specularReflectance" value="{rgb(m[4:7])}"/><float name="intIOR" value="{float(m[7])!r}"/>'
                f'</bsdf>')
    if t == scenes.MAT_ROUGH_DIELECTRIC:
        dist = "ggx" if m[3] else "beckmann"
        return (f'<bsdf type="roughdielectric" id="{ident}"><rgb name="specularReflectance" value="1 1 1"/>'
                f'<rgb name="specularTransmittance" value="1 1 1"/><float name="alpha" value="{float(m[1])!r}"/>'
                f'<float name="intIOR" value="{float(m[2])!r}"/><string name="distribution" value="{dist}"/></bsdf>')
    raise ValueError(t)


def scene_to_files(sc, folder, integrator="path"):
    """The scene as an XML file plus one PLY per run of triangles that share material
    and emission; returns the XML path."""
    os.makedirs(folder, exist_ok=True)
    mats = [bsdf_xml(m, f"m{k}") for k, m in enumerate(sc.materials)]
    emit = sc.tri_emit if sc.tri_emit is not None else np.zeros((sc.ntri, 3), np.float32)
    shapes, start = [], 0
    for i in range(1, sc.ntri + 1):
        if i == sc.ntri or sc.tri_mat[i] != sc.tri_mat[start] or np.any(emit[i] != emit[start]):
            V = sc.verts[start:i].reshape(-1, 3)
            name = f"part{len(shapes)}.ply"
            write_ply(os.path.join(folder, name), V, [[3 * k, 3 * k + 1, 3 * k + 2] for k in range(i - start)])
            em = ""
            if np.any(emit[start] != 0):
                em = f'<emitter type="area"><rgb name="radiance" value="{rgb(emit[start])}"/></emitter>'
            shapes.append(f'<shape type="ply"><string name="filename" value="{name}"/>'
                          f'<ref id="m{int(sc.tri_mat[start])}"/>{em}</shape>')
            start = i
    eye, look, up, fov = sc.camera[:3], sc.camera[3:6], sc.camera[6:9], sc.camera[9]
    xml = f"""<?xml version="1.0" encoding="utf-8"?>
<!-- {sc.name}, written by the scene-file tests -->
<scene version="0.5.0">
  <integrator type="{integrator}"><integer name="maxDepth" value="{sc.max_depth}"/></integrator>
  <sensor type="perspective">
    <float name="fov" value="{float(fov)!r}"/>
    <transform name="toWorld">
      <lookAt origin="{rgb(eye)}" target="{rgb(look)}" up="{rgb(up)}"/>
    </transform>
    <sampler type="independent"><integer name="sampleCount" value="{sc.spp}"/></sampler>
    <film type="hdrfilm">
      <integer name="width" value="{sc.width}"/>
      <integer name="height" value="{sc.height}"/>
      <rfilter type="box"/>
    </film>
  </sensor>
  {''.join(mats)}
  {''.join(shapes)}
</scene>
"""
    path = os.path.join(folder, "scene.xml")
    with open(path, "w") as f:
        f.write(xml)
    return path


def test_box_room_scene_file_reads_back(tmp_path):
    sc = scenes.box_room(width=40, height=30, spp=16, max_depth=7)
    got, integ = load_scene(scene_to_files(sc, tmp_path / "box"))
    assert integ == "path"
    assert (got.width, got.height, got.spp, got.max_depth) == (40, 30, 16, 7)
    np.testing.assert_array_equal(got.verts, sc.verts)
    np.testing.assert_array_equal(got.materials[got.tri_mat].astype(np.float32),
                                  np.asarray(sc.materials)[sc.tri_mat].astype(np.float32))
    np.testing.assert_array_equal(got.tri_emit, sc.tri_emit)
    # camera: the eye, the unit view direction and an up vector in the same plane
    cam = np.asarray(sc.camera, np.float64)
    np.testing.assert_array_equal(got.camera[:3], cam[:3].astype(np.float32))
    d0 = cam[3:6] - cam[:3]
    np.testing.assert_allclose(got.camera[3:6] - got.camera[:3], d0 / np.linalg.norm(d0), atol=1e-6)
    assert abs(np.dot(got.camera[6:9], d0)) < 1e-6 and got.camera[9] == np.float32(cam[9])
    assert got.env is None


def test_material_room_scene_file_reads_back(tmp_path):
    sc = scenes.material_room(width=24, height=24)
    got, integ = load_scene(scene_to_files(sc, tmp_path / "mat", integrator="directlighting"))
    assert integ == "direct"
    np.testing.assert_array_equal(got.verts, sc.verts)
    np.testing.assert_allclose(got.materials[got.tri_mat], np.asarray(sc.materials)[sc.tri_mat], rtol=1e-6)


def _ref():
    from oracle import spo
    if not os.path.isdir(spo.REF_TREE):
        pytest.skip("reference tree not present on this host")
    spo.build("ref")
    return spo.Oracle("ref")


def test_ply_and_transforms_match_reference_bit_for_bit(tmp_path):
    """meshio::loadPLY plus the parser's transform composition (a chain of every
    element kind, rotate angle in radians as the reference reads it)."""
    ref = _ref()
    rng = np.random.default_rng(4)
    V = rng.normal(size=(40, 3)).astype(np.float32)
    faces = [list(rng.choice(40, 3, replace=False)) for _ in range(30)]
    faces += [[0, 1, 2, 3], [4, 5, 6, 7, 8]]   # polygons: the reference keeps their first triangle
    write_ply(tmp_path / "m.ply", V, faces)
    M = rng.normal(size=16)
    chain = [(0, [0.5, -1.25, 3.0]), (2, [0.7, 0.2, 1.0, -0.4]), (1, [2.0, 0.5, 1.5]),
             (3, [1.0, 2.0, 3.0, 0.1, -0.3, 0.2, 0.0, 1.0, 0.1]), (4, list(M)), (2, [-1.3, 0.0, 0.0, 1.0])]
    kinds = [k for k, _ in chain]
    params = np.zeros((len(chain), 16))
    for i, (_, q) in enumerate(chain):
        params[i, :len(q)] = q
    elems = []
    for k, q in chain:
        f = [repr(float(x)) for x in q]
        if k == 0:
            elems.append(f'<translate x="{f[0]}" y="{f[1]}" z="{f[2]}"/>')
        elif k == 1:
            elems.append(f'<scale x="{f[0]}" y="{f[1]}" z="{f[2]}"/>')
        elif k == 2:
            elems.append(f'<rotate angle="{f[0]}" x="{f[1]}" y="{f[2]}" z="{f[3]}"/>')
        elif k == 3:
            elems.append(f'<lookAt origin="{f[0]}, {f[1]}, {f[2]}" target="{f[3]}, {f[4]}, {f[5]}" '
                         f'up="{f[6]}, {f[7]}, {f[8]}"/>')
        else:
            elems.append(f'<matrix value="{" ".join(f)}"/>')
    xml = f"""<scene version="0.5.0"><integrator type="path"/>
<sensor type="perspective"><float name="fov" value="40"/><transform name="toWorld"><lookAt origin="0 0 -5"
target="0 0 0" up="0 1 0"/></transform><sampler type="independent"><integer name="sampleCount" value="4"/></sampler>
<film type="hdrfilm"><integer name="width" value="8"/><integer name="height" value="8"/></film></sensor>
<shape type="ply"><string name="filename" value="m.ply"/><transform name="toWorld">{''.join(elems)}</transform>
<bsdf type="diffuse"><rgb name="reflectance" value="0.5, 0.5, 0.5"/></bsdf></shape></scene>"""
    (tmp_path / "s.xml").write_text(xml)
    got, _ = load_scene(tmp_path / "s.xml")
    T = ref.transform_chain(kinds, params)
    want = ref.load_ply(tmp_path / "m.ply", T)
    assert got.verts.shape == want.shape == (32, 9)
    np.testing.assert_array_equal(got.verts, want.astype(np.float32))


def test_hdr_reader_matches_reference(tmp_path):
    """A Radiance file in the reference's own layout (spgpu_write_hdr) read by
    Image::loadHdr and by spgpu_load_hdr: the same floats, including the reference's
    mantissa * 2^(e-128) / 256 for exponent 0."""
    ref = _ref()
    rng = np.random.default_rng(8)
    px = rng.integers(0, 256, (9, 131, 4)).astype(np.uint8)
    px[0, :4] = [[0, 0, 0, 0], [255, 255, 255, 255], [1, 2, 3, 128], [7, 7, 7, 7]]
    write_hdr(tmp_path / "env.hdr", px)
    got = load_hdr(tmp_path / "env.hdr")
    want = ref.load_hdr(tmp_path / "env.hdr")
    assert got.shape == want.shape == (9, 131, 3)
    np.testing.assert_array_equal(got, want.astype(np.float32))


def _minimal(shapes, extra=""):
    return f"""<scene version="0.5.0"><integrator type="path"><integer name="maxDepth" value="5"/></integrator>
<sensor type="perspective"><float name="fov" value="40"/><transform name="toWorld"><lookAt origin="0 0 -5"
target="0 0 0" up="0 1 0"/></transform><sampler type="independent"><integer name="sampleCount" value="4"/></sampler>
<film type="ldrfilm"><integer name="width" value="8"/><integer name="height" value="6"/></film></sensor>
{extra}{shapes}</scene>"""


def test_parameter_store_rules(tmp_path):
    """The reference's store: a shape consumes the pending bsdf (a later shape without
    one is black) and its toWorld; area-light radiance is read without removal, so a
    later area emitter without its own radiance reuses it; <ref> re-binds an id."""
    write_ply(tmp_path / "t.ply", [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])
    shapes = """
<bsdf type="diffuse" id="red"><rgb name="reflectance" value="0.8 0.1 0.1"/></bsdf>
<shape type="ply"><string name="filename" value="t.ply"/><ref id="red"/>
  <transform name="toWorld"><translate x="0" y="0" z="1"/></transform>
  <emitter type="area"><rgb name="radiance" value="4 5 6"/></emitter></shape>
<shape type="ply"><string name="filename" value="t.ply"/></shape>
<shape type="ply"><string name="filename" value="t.ply"/><ref id="red"/><emitter type="area"/></shape>"""
    (tmp_path / "s.xml").write_text(_minimal(shapes))
    got, _ = load_scene(tmp_path / "s.xml")
    assert got.verts.shape == (3, 9)
    np.testing.assert_array_equal(got.verts[0, 2::3], [1, 1, 1])     # translated
    np.testing.assert_array_equal(got.verts[1, 2::3], [0, 0, 0])     # toWorld was consumed
    M = got.materials[got.tri_mat]
    np.testing.assert_allclose(M[0, :4], [0, 0.8, 0.1, 0.1], rtol=1e-6)
    np.testing.assert_array_equal(M[1], np.zeros(8))                 # bsdf consumed: black
    np.testing.assert_allclose(M[2, :4], [0, 0.8, 0.1, 0.1], rtol=1e-6)
    np.testing.assert_array_equal(got.tri_emit, [[4, 5, 6], [0, 0, 0], [4, 5, 6]])
    assert (got.width, got.height, got.max_depth, got.spp) == (8, 6, 5, 4)


def test_rough_conductors(tmp_path):
    """roughconductor: Beckmann by default (bsdfs/roughconductor.cc:34), GGX on request;
    alpha defaults to 0.1 and is read without removal, so it persists to the next one."""
    write_ply(tmp_path / "t.ply", [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])
    shapes = """
<shape type="ply"><string name="filename" value="t.ply"/>
  <bsdf type="roughconductor"><rgb name="eta" value="0.2 0.3 0.4"/><rgb name="k" value="3 2 1"/></bsdf></shape>
<shape type="ply"><string name="filename" value="t.ply"/>
  <bsdf type="roughconductor"><float name="alpha" value="0.25"/><string name="distribution" value="ggx"/>
    <rgb name="eta" value="1 1 1"/><rgb name="k" value="2 2 2"/></bsdf></shape>
<shape type="ply"><string name="filename" value="t.ply"/>
  <bsdf type="roughconductor"><rgb name="eta" value="1 1 1"/><rgb name="k" value="2 2 2"/></bsdf></shape>"""
    (tmp_path / "s.xml").write_text(_minimal(shapes))
    got, _ = load_scene(tmp_path / "s.xml")
    M = got.materials[got.tri_mat]
    np.testing.assert_allclose(M[0], [scenes.MAT_CONDUCTOR_BECKMANN, 0.1, 0.2, 0.3, 0.4, 3, 2, 1], rtol=1e-6)
    np.testing.assert_allclose(M[1], [scenes.MAT_CONDUCTOR, 0.25, 1, 1, 1, 2, 2, 2], rtol=1e-6)
    np.testing.assert_allclose(M[2], [scenes.MAT_CONDUCTOR_BECKMANN, 0.25, 1, 1, 1, 2, 2, 2], rtol=1e-6)


def test_obj_meshes(tmp_path):
    """OBJ: positions with /texcoord/normal parts ignored, negative (relative) indices,
    polygons as fans around their first vertex."""
    (tmp_path / "q.obj").write_text("# quad and triangle\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\n"
                                    "f 1//1 2//1 3//1 4//1\nv 2 2 2\nf -1 -2 -3\n")
    (tmp_path / "s.xml").write_text(_minimal('<shape type="obj"><string name="filename" value="q.obj"/></shape>'))
    got, _ = load_scene(tmp_path / "s.xml")
    np.testing.assert_array_equal(got.verts, [[0, 0, 0, 1, 0, 0, 1, 1, 0], [0, 0, 0, 1, 1, 0, 0, 1, 0],
                                              [2, 2, 2, 0, 1, 0, 1, 1, 0]])


@pytest.mark.parametrize("snippet, message", [
    ('<bsdf type="conductor" id="c"/><shape type="ply"><string name="filename" value="t.ply"/></shape>',
     "no GPU counterpart"),
    ('<bsdf type="roughconductor"><rgb name="eta" value="1 1 1"/><rgb name="k" value="2 2 2"/>'
     '<string name="distribution" value="phong"/></bsdf>'
     '<shape type="ply"><string name="filename" value="t.ply"/></shape>', "unknown distribution"),
    ('<shape type="sphere"><float name="radius" value="1"/></shape>', "not created by the reference"),
    ('<shape type="ply"><string name="filename" value="missing.ply"/></shape>', "cannot open"),
    ('<medium type="homogeneous"/>', "not supported"),
    ('<shape type="ply"><string name="filename" value="t.ply"/>', "does not close"),
])
def test_refusals(tmp_path, snippet, message):
    write_ply(tmp_path / "t.ply", [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])
    (tmp_path / "s.xml").write_text(_minimal(snippet))
    with pytest.raises(SpgpuError, match=message):
        load_scene(tmp_path / "s.xml")


def test_missing_sample_count_is_refused(tmp_path):
    xml = _minimal("").replace('<integer name="sampleCount" value="4"/>', "")
    (tmp_path / "s.xml").write_text(xml)
    with pytest.raises(SpgpuError, match="sampleCount"):
        load_scene(tmp_path / "s.xml")


def test_headers_that_overstate_the_data_are_refused(tmp_path):
    """A PLY header whose counts the file cannot hold, and an .hdr size line beyond what
    the format encodes, are refused with a message before anything is allocated for
    them (no exception or abort crosses the C ABI)."""
    write_ply(tmp_path / "t.ply", [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]])
    data = (tmp_path / "t.ply").read_bytes()
    (tmp_path / "big.ply").write_bytes(data.replace(b"element vertex 3", b"element vertex 1000000000000"))
    (tmp_path / "faces.ply").write_bytes(data.replace(b"element face 1", b"element face 2"))
    for name in ("big.ply", "faces.ply"):
        (tmp_path / "s.xml").write_text(_minimal(f'<shape type="ply"><string name="filename" value="{name}"/></shape>'))
        with pytest.raises(SpgpuError, match="exceed the file"):
            load_scene(tmp_path / "s.xml")
    (tmp_path / "huge.hdr").write_bytes(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 2000000000 +X 30000\n")
    with pytest.raises(SpgpuError, match="too large"):
        load_hdr(tmp_path / "huge.hdr")


def _mutate(data, rng):
    b = bytearray(data)
    for _ in range(int(rng.integers(1, 7))):
        op, i = rng.random(), int(rng.integers(0, len(b) + 1))
        if op < 0.4 and b:
            b[min(i, len(b) - 1)] = int(rng.integers(0, 256))
        elif op < 0.6:
            b[i:i] = bytes([int(rng.integers(0, 256))])
        elif op < 0.8 and b:
            del b[min(i, len(b) - 1)]
        else:
            del b[i:]
    return bytes(b)


def test_malformed_files_are_refused_not_crashed(tmp_path):
    """Seeded byte-level mutations of a scene file, a PLY mesh and an .hdr map: every
    load either succeeds or raises SpgpuError with a message (the message may quote
    bytes of the file).  Nothing reads out of bounds or aborts the process."""
    rng = np.random.default_rng(2024)
    write_ply(tmp_path / "base.ply", rng.random((30, 3)), [[i, (i + 1) % 30, (i + 2) % 30] for i in range(30)])
    write_hdr(tmp_path / "base.hdr", rng.integers(0, 255, (5, 9, 4)).astype(np.uint8))
    xml = _minimal('<shape type="ply"><string name="filename" value="base.ply"/>'
                   '<emitter type="area"><rgb name="radiance" value="1 2 3"/></emitter></shape>')
    ply, hdr = (tmp_path / "base.ply").read_bytes(), (tmp_path / "base.hdr").read_bytes()
    outcomes = {"loaded": 0, "refused": 0}
    for k in range(450):
        kind = k % 3
        if kind == 0:
            (tmp_path / "m.xml").write_bytes(_mutate(xml.encode(), rng))
            call = lambda: load_scene(tmp_path / "m.xml")   # noqa: E731
        elif kind == 1:
            (tmp_path / "m.ply").write_bytes(_mutate(ply, rng))
            (tmp_path / "m.xml").write_text(_minimal('<shape type="ply"><string name="filename" value="m.ply"/></shape>'))
            call = lambda: load_scene(tmp_path / "m.xml")   # noqa: E731
        else:
            (tmp_path / "m.hdr").write_bytes(_mutate(hdr, rng))
            call = lambda: load_hdr(tmp_path / "m.hdr")   # noqa: E731
        try:
            call()
            outcomes["loaded"] += 1
        except SpgpuError as e:
            assert str(e), k
            outcomes["refused"] += 1
    assert outcomes["loaded"] > 20 and outcomes["refused"] > 20, outcomes
