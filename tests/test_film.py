"""Film output on the host (no GPU): the .hdr writer reproduces the compiled
reference's file (Image::saveHdr, core/image.cc:390) byte for byte from the same RGBE
pixels, the RGBE pixels themselves follow the reference's HDRPixel rule
(core/image.cc:72-88) restated here in numpy, and the PNG writer round-trips."""
import os
import struct
import zlib

import numpy as np
import pytest

from conftest import GOLDEN


def parse_hdr(data: bytes):
    """(W, H, RGBE pixels) of a file in Image::saveHdr's layout."""
    i = data.index(b"\n-Y ")
    j = data.index(b"\n", i + 1)
    _, H, _, W = data[i + 1:j].split()
    H, W = int(H), int(W)
    p = j + 1
    px = np.zeros((H, W, 4), np.uint8)
    for y in range(H):
        assert data[p:p + 2] == b"\x02\x02" and (data[p + 2] << 8 | data[p + 3]) == W
        p += 4
        for c in range(4):
            x = 0
            while x < W:
                n = data[p]
                assert 0 < n <= 127
                px[y, x:x + n, c] = np.frombuffer(data[p + 1:p + 1 + n], np.uint8)
                p += 1 + n
                x += n
    assert p == len(data)
    return W, H, px


def rgbe_numpy(film):
    """HDRPixel of Film::save's resolve, restated (float64 like the reference)."""
    c = film[..., :3].astype(np.float64) / (film[..., 3:4].astype(np.float64) + 1e-12)
    d = c.max(-1)
    m, e = np.frexp(d)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = m * 256.0 / d
    out = np.zeros(film.shape[:2] + (4,), np.uint8)
    ok = d > 1e-32
    out[ok, :3] = (c[ok] * s[ok, None]).astype(np.uint8)
    out[ok, 3] = (e[ok] + 128).astype(np.uint8)
    return out


def test_hdr_writer_reproduces_reference_file(tmp_path):
    from spica_gb300 import gpu
    g = np.load(os.path.join(GOLDEN, "film_output.npz"))
    ref = bytes(g["hdr"])
    W, H, px = parse_hdr(ref)
    assert (H, W) == g["film"].shape[:2]
    path = tmp_path / "out.hdr"
    gpu.write_hdr(str(path), px)
    assert path.read_bytes() == ref


def test_rgbe_rule_matches_reference_pixels():
    g = np.load(os.path.join(GOLDEN, "film_output.npz"))
    _, _, px = parse_hdr(bytes(g["hdr"]))
    np.testing.assert_array_equal(rgbe_numpy(g["film"]), px)


def test_png_writer_round_trip(tmp_path):
    from spica_gb300 import gpu
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, (23, 70000 // 69, 3), dtype=np.uint8)   # > 64 KiB of scanlines: several blocks
    path = tmp_path / "out.png"
    gpu.write_png(str(path), img)
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    p, chunks = 8, {}
    while p < len(data):
        n, = struct.unpack(">I", data[p:p + 4])
        typ, body = data[p + 4:p + 8], data[p + 8:p + 8 + n]
        crc, = struct.unpack(">I", data[p + 8 + n:p + 12 + n])
        assert crc == zlib.crc32(typ + body)
        chunks[typ] = body
        p += 12 + n
    W, H, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    assert (W, H, depth, ctype) == (img.shape[1], img.shape[0], 8, 2)
    raw = np.frombuffer(zlib.decompress(chunks[b"IDAT"]), np.uint8).reshape(H, 3 * W + 1)
    assert not raw[:, 0].any()
    np.testing.assert_array_equal(raw[:, 1:].reshape(img.shape), img)


def test_tone_mapping_restatement_matches_reference():
    """The numpy restatement of ReinhardTmo, DragoTmo and DurandTMO (oracle/tmo_oracle.py),
    which checks the device operators, against the compiled reference's images."""
    from oracle import tmo_oracle
    g = np.load(os.path.join(GOLDEN, "film_output.npz"))
    np.testing.assert_allclose(tmo_oracle.reinhard(g["film"], 0.18), g["reinhard"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(tmo_oracle.drago(g["film"], 0.85), g["drago"], rtol=1e-13, atol=0)
    durand = tmo_oracle.durand(g["film"], 5.0)
    np.testing.assert_allclose(durand, g["durand"], rtol=1e-13, atol=1e-15)
    inside = (g["durand"] > 0) & (g["durand"] < 1)
    assert inside.mean() > 0.5   # the image is mostly not clipped: the comparison means something


@pytest.mark.parametrize("H, W", [(1, 1), (1, 9), (7, 1), (48, 64)])
def test_tone_mapping_restatement_on_random_films(ref, H, W):
    """The numpy restatement against the compiled reference's operators on seeded films,
    including single-row and single-column images (the bilateral filter's scans have
    nothing to do along a unit dimension) and black pixels."""
    from oracle import tmo_oracle
    rng = np.random.default_rng(H * 1000 + W)
    film = np.empty((H, W, 4), np.float32)
    film[..., :3] = rng.lognormal(0.0, 2.0, (H, W, 3)).astype(np.float32)
    film[..., 3] = rng.integers(1, 64, (H, W)).astype(np.float32)
    film[rng.random((H, W)) < 0.1] = 0.0
    np.testing.assert_allclose(tmo_oracle.reinhard(film, 0.3), ref.film_reinhard(film, 0.3), rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(tmo_oracle.drago(film, 0.7), ref.film_drago(film, 0.7), rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(tmo_oracle.durand(film, 4.0), ref.film_durand(film, 4.0), rtol=1e-12, atol=1e-15)
