"""Output side of the path: tonemapper and film writers (host code; the GPU
tonemapper is checked in tests/test_gpu_render.py)."""
import struct
import zlib

import numpy as np
import pytest

from oracle.binding import tonemap as oracle_tonemap
from renderer_gb300.output import tonemap, write_image
from renderer_gb300.scenefile import read_hdr

pytestmark = pytest.mark.usefixtures("gbrt_built")


def film(h=7, w=5, seed=0):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0, 1.5, (h, w, 3)).astype(np.float32)
    f[0, 0] = (0, 0, 0)
    f[0, 1] = (np.nan, -1, 300)
    return f


def test_tonemap_matches_the_renderer_formula():
    f = film()
    got = tonemap(f, 2.2)
    np.testing.assert_array_equal(got, oracle_tonemap(f, 2.2))
    # clamp(255 * c^(1/2.2)) truncated, BGR -> RGB
    c = float(f[3, 2, 0])
    assert got[3, 2, 2] == min(255, int(np.float32(255 * c ** (1 / 2.2))))
    assert list(got[0, 1]) == [255, 0, 0]   # R = 300 saturates, G < 0 and B = NaN give 0


def test_exr_layout(tmp_path):
    f = film(4, 3)
    p = str(tmp_path / "a.exr")
    write_image(p, f)
    b = open(p, "rb").read()
    assert struct.unpack("<II", b[:8]) == (20000630, 2)
    i = 8
    attrs = {}
    while b[i] != 0:
        n = b.index(b"\0", i); name = b[i:n].decode(); i = n + 1
        n = b.index(b"\0", i); typ = b[i:n].decode(); i = n + 1
        size = struct.unpack("<i", b[i:i + 4])[0]; i += 4
        attrs[name] = (typ, b[i:i + size]); i += size
    i += 1
    assert attrs["compression"] == ("compression", b"\0")
    assert struct.unpack("<4i", attrs["dataWindow"][1]) == (0, 0, 2, 3)
    offsets = struct.unpack("<4Q", b[i:i + 32])
    for y, off in enumerate(offsets):
        yy, size = struct.unpack("<ii", b[off:off + 8])
        assert yy == y and size == 3 * 3 * 4
        data = np.frombuffer(b[off + 8:off + 8 + size], np.float32).reshape(3, 3)   # B, G, R planes
        np.testing.assert_array_equal(data.T, f[y])


def test_pfm_hdr_m(tmp_path):
    f = np.abs(film(6, 4)); f[0, 1] = (0.5, 2.0, 3.0)
    write_image(str(tmp_path / "a.pfm"), f)
    np.testing.assert_array_equal(read_hdr(str(tmp_path / "a.pfm")), f)
    write_image(str(tmp_path / "a.hdr"), f)
    back = read_hdr(str(tmp_path / "a.hdr"))
    assert np.all(np.abs(back - f) <= f.max(-1, keepdims=True) / 128.0 + 1e-30)
    write_image(str(tmp_path / "im1.m"), f)
    txt = open(tmp_path / "im1.m").read()
    assert txt.startswith("function im = im1()\n  im = zeros(6,4,3);\n")
    assert txt.count("im(:, :, ") == 3 and txt.rstrip().endswith("end")


def test_png_bmp_ppm(tmp_path):
    f = film(9, 11)
    rgb = tonemap(f, 2.2)
    write_image(str(tmp_path / "a.png"), f)
    b = open(tmp_path / "a.png", "rb").read()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    i, idat = 8, b""
    while i < len(b):
        n = struct.unpack(">I", b[i:i + 4])[0]
        typ, data = b[i + 4:i + 8], b[i + 8:i + 8 + n]
        assert zlib.crc32(typ + data) == struct.unpack(">I", b[i + 8 + n:i + 12 + n])[0]
        if typ == b"IDAT":
            idat += data
        i += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(9, 1 + 11 * 3)
    assert np.all(raw[:, 0] == 0)
    np.testing.assert_array_equal(raw[:, 1:].reshape(9, 11, 3), rgb)
    write_image(str(tmp_path / "a.ppm"), f)
    p = open(tmp_path / "a.ppm", "rb").read()
    assert p.startswith(b"P6\n11 9\n255\n")
    np.testing.assert_array_equal(np.frombuffer(p[len(b"P6\n11 9\n255\n"):], np.uint8).reshape(9, 11, 3), rgb)
    write_image(str(tmp_path / "a.bmp"), f)
    m = open(tmp_path / "a.bmp", "rb").read()
    assert m[:2] == b"BM" and struct.unpack("<ii", m[18:26]) == (11, 9)
    row = (11 * 3 + 3) & ~3
    px = np.frombuffer(m[54:], np.uint8).reshape(9, row)[:, :33].reshape(9, 11, 3)[::-1, :, ::-1]
    np.testing.assert_array_equal(px, rgb)
