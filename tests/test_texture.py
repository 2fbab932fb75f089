"""TextureMaterial (src/texturematerial.cpp:33-74): a diffuse material whose
albedo is pow(kd * bilinear(texture, uv), gamma), uv interpolated over
triangles from their texture coordinates (default (0,0), (0,1), (1,0)).

CPU: the oracle against closed forms (a constant texture is a diffuse
material; a textured floor under a point light shows the texel values), the
parser (texture(...) reads PPM, PNG and JPEG, scales by 1/255, unreadable files give
DarkMatter). GPU: path-level parity with the oracle on a scene whose texture
varies across the image, for both estimators."""
import math
import os

import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import _abi
from renderer_gb300.scene import SceneData, render_params


def floor_scene(tex, kd=(1.0, 1.0, 1.0), gamma=1.0, uv=None, width=16):
    """A textured floor quad made of two triangles under a point light and a
    camera looking straight down."""
    s = SceneData()
    t = s.add_texture(tex)
    m = s.add_material(_abi.MAT_TEXTURE, kd=kd, exponent=gamma, texture=t)
    a, b, c, d = (-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)
    s.tri_pos = np.array([a + b + c, a + c + d], np.float32)
    s.tri_mat = np.array([m, m], np.int32)
    if uv is not None:
        s.tri_uv = np.asarray(uv, np.float32)
    s.lights = [dict(type=_abi.LIGHT_POINT, origin=(0, 2, 0), intensity=(4, 4, 4))]
    s.camera = dict(eye=(0, 3, 0.0001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.5, width=width, height=width)
    return s


def checker(n=8):
    y, x = np.mgrid[0:n, 0:n]
    v = ((x + y) % 2).astype(np.float32) * 0.8 + 0.1
    return np.stack([v, 0.5 * v, np.full_like(v, 0.3)], -1)


def test_constant_texture_is_diffuse():
    """A constant texture equals DiffuseMaterial with that colour (times kd,
    to the power gamma), pixel for pixel with the same random numbers."""
    tex = np.full((4, 4, 3), 0.5, np.float32)
    a = floor_scene(tex, kd=(0.8, 0.6, 0.4), gamma=2.0)
    b = floor_scene(tex)
    b.materials[0] = dict(type=_abi.MAT_DIFFUSE, kd=(0.4 ** 2, 0.3 ** 2, 0.2 ** 2), ks=(0, 0, 0), exponent=0.0,
                          ior=1.0, coefficient=1.0, texture=-1)
    p = render_params(2, 2, 0.5, 4, 3)
    fa = OracleScene(a).render(a.camera_struct(), p, rng_mode=1)["film"]
    fb = OracleScene(b).render(b.camera_struct(), p, rng_mode=1)["film"]
    np.testing.assert_allclose(fa, fb, rtol=2e-6, atol=1e-9)


def test_texture_lookup_follows_uv():
    """With explicit uv the image under the light is the texture itself, up
    to the point light's 1/r^2 cos falloff (a pure NEE scene, depth 1)."""
    tex = checker(8)
    uv = [[0, 1, 1, 1, 1, 0], [0, 1, 1, 0, 0, 0]]  # (u, v) = ((x+1)/2, (1-z)/2)
    s = floor_scene(tex, uv=uv, width=32)
    r = OracleScene(s).render(s.camera_struct(), render_params(1, 1, 0.0, 1, 0), rng_mode=1)["film"]
    lit = r[..., 1] > 0
    assert lit.mean() > 0.9
    # channel 0 of the checker is twice channel 1 in every texel, hence in
    # every bilinear sample: the ratio survives shading; channel 0 varies.
    np.testing.assert_allclose(r[..., 0][lit] / r[..., 1][lit], 2.0, rtol=1e-5)
    assert r[..., 0].std() > 0.1 * r[..., 0].mean()


def test_parser_reads_ppm_texture(tmp_path):
    from renderer_gb300.scenefile import load_scene_string
    img = (np.arange(2 * 3 * 3) * 10).astype(np.uint8).reshape(2, 3, 3)
    p = tmp_path / "t.ppm"
    p.write_bytes(b"P6\n3 2\n255\n" + img.tobytes())
    s = load_scene_string('intersectable = intersectables { t([0 0 0], [1 0 0], [0 1 0], [0 0 1], [0 0 1], '
                          '[0 0 1], [0 0], [1 0], [0 1], texture("t.ppm", [1 0.5 0.25], 2.2)) };', str(tmp_path))
    m = s.materials[0]
    assert m["type"] == _abi.MAT_TEXTURE and m["exponent"] == pytest.approx(2.2)
    assert m["kd"] == pytest.approx((0.25, 0.5, 1.0))  # BGR
    np.testing.assert_allclose(s.textures[m["texture"]], img[..., ::-1] / 255.0, rtol=1e-6)
    np.testing.assert_allclose(s.tri_uv[0], [0, 0, 1, 0, 0, 1])
    missing = load_scene_string('intersectable = intersectables { sphere([0 0 0], 1, '
                                'texture("nope.ppm", [1 1 1], 1)) };', str(tmp_path))
    assert missing.materials[0]["type"] == _abi.MAT_DARK


# ------------------------------------------------------------------ GPU ----
def textured_room():
    """The Cornell box with a checker texture on the back wall and floor."""
    from renderer_gb300 import workloads
    s = workloads.cornell_box(64, 64)
    t = s.add_texture(checker(16))
    m = s.add_material(_abi.MAT_TEXTURE, kd=(1, 1, 1), exponent=1.0, texture=t)
    floor, back = s.quads[0], s.quads[2]
    tris, uvs = [], []
    for q, rep in ((floor, 2.0), (back, 3.0)):
        p1, p2, p3, p4 = [np.array(v, np.float32) for v in q[:4]]
        tris += [np.concatenate([p1, p2, p3]), np.concatenate([p1, p3, p4])]
        uvs += [[0, 0, rep, 0, rep, rep], [0, 0, rep, rep, 0, rep]]
    s.quads = [q for i, q in enumerate(s.quads) if i not in (0, 2)]
    c, r, _ = s.spheres[0]
    s.spheres[0] = (c, r, m)  # a textured sphere (spherical texture coordinates)
    s.tri_pos = np.array(tris, np.float32)
    s.tri_uv = np.array(uvs, np.float32)
    s.tri_mat = np.full(len(tris), m, np.int32)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("semantics", [_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL])
def test_textured_path_level_parity(ctx, semantics):
    from renderer_gb300.runtime import GpuScene
    from tests.test_gpu_render import gpu_render
    s = textured_room()
    prm = render_params(2, 2, 0.5, 6, 9, semantics=semantics)
    (film, _, _), _ = gpu_render(ctx, s, prm)
    orc = OracleScene(s).render(s.camera_struct(), prm, rng_mode=1)["film"]
    close = np.isclose(film, orc, rtol=2e-3, atol=1e-5).all(-1)
    assert close.mean() > 0.97, close.mean()
    assert film.mean() == pytest.approx(orc.mean(), rel=5e-3)


# ------------------------------------------------------------------ PNG ----
# An independent PNG writer (Python's zlib for DEFLATE, the filters and Adam7
# written out here) feeds the library's decoder; the expected image is what
# cv::imread(IMREAD_COLOR) gives: 8-bit BGR, grey replicated, palette
# expanded, alpha dropped, 16-bit samples reduced to their high byte.
import struct
import zlib

_ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
_CHANS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(t, body):
    return struct.pack(">I", len(body)) + t + body + struct.pack(">I", zlib.crc32(t + body) & 0xFFFFFFFF)


def _pack_rows(samples, depth):
    """(h, w, c) integer samples -> list of packed row byte strings."""
    h, w, c = samples.shape
    rows = []
    for y in range(h):
        flat = samples[y].reshape(-1).astype(np.int64)
        if depth == 16:
            rows.append(flat.astype(">u2").tobytes())
        elif depth == 8:
            rows.append(flat.astype(np.uint8).tobytes())
        else:
            per = 8 // depth
            pad = (-len(flat)) % per
            f = np.concatenate([flat, np.zeros(pad, np.int64)]).reshape(-1, per)
            shifts = np.array([8 - depth * (k + 1) for k in range(per)])
            rows.append((f << shifts).sum(1).astype(np.uint8).tobytes())
    return rows


def _filter_rows(rows, bpp, rng):
    """Applies a random PNG filter (0-4) to each row; returns the filtered stream."""
    out = bytearray()
    prev = bytes(len(rows[0])) if rows else b""
    for r in rows:
        f = int(rng.integers(0, 5))
        x, b = np.frombuffer(r, np.uint8).astype(np.int64), np.frombuffer(prev, np.uint8).astype(np.int64)
        a = np.concatenate([np.zeros(bpp, np.int64), x[:-bpp]]) if len(x) > bpp else np.zeros_like(x)
        c = np.concatenate([np.zeros(bpp, np.int64), b[:-bpp]]) if len(x) > bpp else np.zeros_like(x)
        if f == 0:
            pred = np.zeros_like(x)
        elif f == 1:
            pred = a
        elif f == 2:
            pred = b
        elif f == 3:
            pred = (a + b) >> 1
        else:
            p = a + b - c
            pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
        out.append(f)
        out += ((x - pred) & 255).astype(np.uint8).tobytes()
        prev = r
    return bytes(out)


def write_png(path, samples, depth, ctype, palette=None, interlace=False, seed=0, level=6,
              strategy=zlib.Z_DEFAULT_STRATEGY, split_idat=1):
    h, w, c = samples.shape
    assert c == _CHANS[ctype]
    rng = np.random.default_rng(seed)
    bpp = max(1, c * depth // 8)
    raw = b""
    for (x0, y0, dx, dy) in (_ADAM7 if interlace else [(0, 0, 1, 1)]):
        sub = samples[y0::dy, x0::dx]
        if sub.size:
            raw += _filter_rows(_pack_rows(sub, depth), bpp, rng)
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy)
    z = co.compress(raw) + co.flush()
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    png += _chunk(b"tEXt", b"Comment\x00ancillary chunk")
    if palette is not None:
        png += _chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    step = -(-len(z) // split_idat)
    for k in range(0, len(z), step):
        png += _chunk(b"IDAT", z[k:k + step])
    png += _chunk(b"IEND", b"")
    path.write_bytes(png)


def imread_color(samples, depth, ctype, palette=None):
    """cv::imread(IMREAD_COLOR) of those samples: (h, w, 3) BGR 0..255."""
    s = samples.astype(np.int64)
    if depth == 16:
        s = s >> 8
    if ctype == 3:
        rgb = np.asarray(palette, np.int64)[s[..., 0]]
    elif ctype in (0, 4):
        g = s[..., 0] * (255 // ((1 << depth) - 1)) if depth < 8 else s[..., 0]
        rgb = np.stack([g, g, g], -1)
    else:
        rgb = s[..., :3]
    return rgb[..., ::-1].astype(np.float32)


PNG_CASES = [(ct, d) for ct, ds in ((0, (1, 2, 4, 8, 16)), (2, (8, 16)), (3, (1, 2, 4, 8)), (4, (8, 16)),
                                    (6, (8, 16))) for d in ds]


@pytest.mark.parametrize("ctype,depth", PNG_CASES)
@pytest.mark.parametrize("interlace", [False, True])
def test_png_decoder_matches_imread_color(tmp_path, ctype, depth, interlace):
    from renderer_gb300.scenefile import read_hdr
    rng = np.random.default_rng(ctype * 100 + depth + 7 * interlace)
    h, w = 13, 11  # odd sizes: partial Adam7 blocks and packed rows with padding bits
    palette = None
    top = (1 << depth) - 1
    if ctype == 3:
        n = min(1 << depth, 40)
        palette = rng.integers(0, 256, (n, 3))
        top = n - 1
    samples = rng.integers(0, top + 1, (h, w, _CHANS[ctype]))
    p = tmp_path / "img.png"
    write_png(p, samples, depth, ctype, palette, interlace, seed=depth, split_idat=3)
    got = read_hdr(str(p))
    np.testing.assert_array_equal(got, imread_color(samples, depth, ctype, palette))


@pytest.mark.parametrize("level,strategy", [(0, zlib.Z_DEFAULT_STRATEGY), (1, zlib.Z_FIXED), (9, zlib.Z_DEFAULT_STRATEGY),
                                            (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE)])
def test_png_deflate_block_kinds(tmp_path, level, strategy):
    """Stored, fixed-Huffman and dynamic-Huffman blocks, long matches and
    overlapping copies (a smooth 300 x 200 RGB image with flat runs)."""
    from renderer_gb300.scenefile import read_hdr
    y, x = np.mgrid[0:200, 0:300]
    img = np.stack([(x // 7) % 256, (y * 3) % 256, ((x + y) // 50) * 40 % 256], -1)
    img[50:90, :, :] = 17  # long runs
    p = tmp_path / "big.png"
    write_png(p, img, 8, 2, level=level, strategy=strategy)
    np.testing.assert_array_equal(read_hdr(str(p)), img[..., ::-1].astype(np.float32))


def test_png_rejects_damage(tmp_path):
    """A flipped byte fails the chunk CRC; a truncated file and a bad zlib
    stream are refused; a scene texture that fails to decode is DarkMatter."""
    from renderer_gb300.scenefile import load_scene_string, read_hdr
    img = np.random.default_rng(3).integers(0, 256, (8, 8, 3))
    p = tmp_path / "ok.png"
    write_png(p, img, 8, 2)
    good = p.read_bytes()
    for bad in (good[:40] + bytes([good[40] ^ 1]) + good[41:], good[:-20]):
        q = tmp_path / "bad.png"
        q.write_bytes(bad)
        with pytest.raises(Exception):
            read_hdr(str(q))
    # a valid CRC around an IDAT whose zlib header is wrong
    ihdr_end = 8 + 25
    body = b"\x78\x9c"[::-1] + zlib.compress(b"\x00" * 10)[2:]
    q = tmp_path / "badz.png"
    q.write_bytes(good[:ihdr_end] + _chunk(b"IDAT", body) + _chunk(b"IEND", b""))
    with pytest.raises(Exception):
        read_hdr(str(q))
    s = load_scene_string('intersectable = intersectables { sphere([0 0 0], 1, texture("bad.png", [1 1 1], 1)) };',
                          str(tmp_path))
    assert s.materials[0]["type"] == _abi.MAT_DARK


def test_parser_reads_png_texture(tmp_path):
    """texture("t.png", ...) in a scene file: the 8-bit image scaled by 1/255,
    like cv::imread + convertTo (src/texturematerial.cpp:48-60)."""
    from renderer_gb300.scenefile import load_scene_string
    img = np.random.default_rng(5).integers(0, 256, (5, 7, 4))
    write_png(tmp_path / "t.png", img, 8, 6, interlace=True)
    s = load_scene_string('intersectable = intersectables { t([0 0 0], [1 0 0], [0 1 0], [0 0 1], [0 0 1], '
                          '[0 0 1], [0 0], [1 0], [0 1], texture("t.png", [1 1 1], 1)) };', str(tmp_path))
    m = s.materials[0]
    assert m["type"] == _abi.MAT_TEXTURE
    np.testing.assert_allclose(s.textures[m["texture"]], img[..., 2::-1] / 255.0, rtol=1e-6)


PNG_FLOOR_SCENE = """
camera = camera([0 3 0.0001], [0 0 0], [0 0 -1], 0.5, 40, 40);
lights = lights { pointlight([0 2 0], [4 4 4]) };
intersectable = intersectables {
  t([-1 0 -1], [1 0 -1], [1 0 1], [0 1 0], [0 1 0], [0 1 0], [0 1], [1 1], [1 0], texture("floor.png", [1 0.9 0.8], 2.2))
  t([-1 0 -1], [1 0 1], [-1 0 1], [0 1 0], [0 1 0], [0 1 0], [0 1], [1 0], [0 0], texture("floor.png", [1 0.9 0.8], 2.2))
};
"""


@pytest.mark.gpu
@pytest.mark.parametrize("semantics", [_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL])
def test_png_textured_scene_parity(ctx, tmp_path, semantics):
    """A scene file with a PNG-textured floor (palette PNG, Adam7): the GPU
    render against the oracle, path by path, on the parsed scene."""
    from renderer_gb300.scenefile import load_scene_string
    from tests.test_gpu_render import gpu_render
    rng = np.random.default_rng(11)
    pal = rng.integers(0, 256, (16, 3))
    write_png(tmp_path / "floor.png", rng.integers(0, 16, (24, 24, 1)), 4, 3, palette=pal, interlace=True)
    s = load_scene_string(PNG_FLOOR_SCENE, str(tmp_path))
    assert s.materials[0]["type"] == _abi.MAT_TEXTURE
    prm = render_params(2, 2, 0.5, 4, 5, semantics=semantics)
    (film, _, _), _ = gpu_render(ctx, s, prm)
    orc = OracleScene(s).render(s.camera_struct(), prm, rng_mode=1)["film"]
    assert film[..., 0].std() > 0.05 * film[..., 0].mean()  # the texture shows
    close = np.isclose(film, orc, rtol=2e-3, atol=1e-5).all(-1)
    assert close.mean() > 0.98, close.mean()


# ----------------------------------------------------------------- JPEG ----
# The decoder against the standard's reconstruction of the same quantised
# coefficients (tests/jpeg_writer.py: exact inverse DCT, triangle-filter
# chroma upsampling, JFIF colour conversion), within one 8-bit unit for the
# rounding of float arithmetic.
def _smooth_rgb(h, w, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    img = np.stack([128 + 100 * np.sin(x / 5.0 + seed), 128 + 90 * np.cos(y / 7.0), (x * 3 + y * 5) % 256], -1)
    img = img + rng.normal(0, 12, img.shape)
    return np.clip(img, 0, 255).astype(np.uint8)


QTABLES = {"fine": np.full(64, 2), "coarse": 4 + np.arange(64) // 2}


@pytest.mark.parametrize("sub,grey", [((2, 2), False), ((2, 1), False), ((1, 1), False), ((1, 1), True)])
@pytest.mark.parametrize("qname", ["fine", "coarse"])
@pytest.mark.parametrize("restart,interleaved", [(0, True), (3, True), (2, False)])
def test_jpeg_decoder_matches_the_standard(tmp_path, sub, grey, qname, restart, interleaved):
    from renderer_gb300.scenefile import read_hdr
    from tests.jpeg_writer import encode, reconstruct
    img = _smooth_rgb(29, 37, seed=len(qname) + restart)
    data, comps, layout = encode(img, QTABLES[qname], subsampling=sub, grey=grey, restart=restart,
                                 interleaved=interleaved)
    p = tmp_path / "t.jpg"
    p.write_bytes(data)
    got = read_hdr(str(p))
    want = reconstruct(comps, layout, grey=grey)
    assert got.shape == want.shape == (29, 37, 3)
    assert np.abs(got - want).max() <= 1.0
    # and, without chroma subsampling and with fine quantisation, close to
    # the image that was encoded (a lossy codec)
    if not grey and qname == "fine" and sub == (1, 1):
        assert np.abs(got[..., ::-1].astype(np.float64) - img).mean() < 3.0


def test_jpeg_refusals(tmp_path):
    """Progressive (SOF2) and truncated files are refused; a texture that
    cannot be read is DarkMatter."""
    from renderer_gb300.scenefile import load_scene_string, read_hdr
    from tests.jpeg_writer import encode
    data, _, _ = encode(_smooth_rgb(16, 16, 1), QTABLES["fine"])
    prog = bytearray(data)
    i = prog.index(b"\xFF\xC0")
    prog[i + 1] = 0xC2
    for bad in (bytes(prog), data[: len(data) // 2], data[:200] + b"\x00" * 50):
        q = tmp_path / "bad.jpg"
        q.write_bytes(bad)
        with pytest.raises(Exception):
            read_hdr(str(q))
    s = load_scene_string('intersectable = intersectables { sphere([0 0 0], 1, texture("bad.jpg", [1 1 1], 1)) };',
                          str(tmp_path))
    assert s.materials[0]["type"] == _abi.MAT_DARK


def test_parser_reads_jpeg_texture(tmp_path):
    from renderer_gb300.scenefile import load_scene_string
    from tests.jpeg_writer import encode, reconstruct
    img = _smooth_rgb(20, 24, 2)
    data, comps, layout = encode(img, QTABLES["fine"])
    (tmp_path / "t.jpeg").write_bytes(data)
    s = load_scene_string('intersectable = intersectables { t([0 0 0], [1 0 0], [0 1 0], [0 0 1], [0 0 1], '
                          '[0 0 1], [0 0], [1 0], [0 1], texture("t.jpeg", [1 1 1], 1)) };', str(tmp_path))
    m = s.materials[0]
    assert m["type"] == _abi.MAT_TEXTURE
    np.testing.assert_allclose(s.textures[m["texture"]] * 255.0, reconstruct(comps, layout), atol=1.0 + 1e-3)


@pytest.mark.gpu
def test_jpeg_textured_scene_parity(ctx, tmp_path):
    """The PNG floor scene with a 4:2:0 JPEG texture: GPU against the oracle
    path by path."""
    from renderer_gb300.scenefile import load_scene_string
    from tests.jpeg_writer import encode
    from tests.test_gpu_render import gpu_render
    data, _, _ = encode(_smooth_rgb(24, 24, 5), QTABLES["coarse"])
    (tmp_path / "floor.png").write_bytes(data)  # the scene names floor.png; the format is found by its bytes
    s = load_scene_string(PNG_FLOOR_SCENE, str(tmp_path))
    assert s.materials[0]["type"] == _abi.MAT_TEXTURE
    prm = render_params(2, 2, 0.5, 4, 6)
    (film, _, _), _ = gpu_render(ctx, s, prm)
    orc = OracleScene(s).render(s.camera_struct(), prm, rng_mode=1)["film"]
    close = np.isclose(film, orc, rtol=2e-3, atol=1e-5).all(-1)
    assert close.mean() > 0.98, close.mean()


def test_png_and_jpeg_edge_sizes(tmp_path):
    """1 x 1 images, an 8 x 8 JPEG (one block exactly), a restart marker after
    every MCU, and an oversized PNG header refused."""
    from renderer_gb300.scenefile import read_hdr
    from tests.jpeg_writer import encode, reconstruct
    one = np.array([[[200, 30, 90, 255]]])
    write_png(tmp_path / "one.png", one, 8, 6)
    np.testing.assert_array_equal(read_hdr(str(tmp_path / "one.png")), [[[90.0, 30.0, 200.0]]])
    for h, w, sub, restart in ((1, 1, (2, 2), 0), (8, 8, (1, 1), 0), (17, 23, (2, 2), 1)):
        img = _smooth_rgb(h, w, h + w)
        data, comps, layout = encode(img, QTABLES["coarse"], subsampling=sub, restart=restart)
        p = tmp_path / ("e%d.jpg" % h)
        p.write_bytes(data)
        got = read_hdr(str(p))
        assert got.shape == (h, w, 3)
        assert np.abs(got - reconstruct(comps, layout)).max() <= 1.0
    big = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", 70000, 2, 8, 2, 0, 0, 0)) + \
        _chunk(b"IEND", b"")
    (tmp_path / "big.png").write_bytes(big)
    with pytest.raises(Exception):
        read_hdr(str(tmp_path / "big.png"))


def test_decoders_survive_damaged_files(tmp_path):
    """Truncated and byte-flipped PNG and JPEG files (seeded): every one is
    either decoded to 8-bit values or refused with an error status, never a
    crash (the decoders also ran clean under AddressSanitizer and UBSan on
    6,000 such files)."""
    from renderer_gb300 import GbrtError
    from renderer_gb300.scenefile import read_hdr
    from tests.jpeg_writer import encode
    rng = np.random.default_rng(12)
    srcs = []
    write_png(tmp_path / "a.png", rng.integers(0, 256, (9, 13, 3)), 8, 2, interlace=True)
    srcs.append((tmp_path / "a.png").read_bytes())
    write_png(tmp_path / "b.png", rng.integers(0, 65536, (6, 7, 4)), 16, 6)
    srcs.append((tmp_path / "b.png").read_bytes())
    srcs.append(encode(_smooth_rgb(21, 19, 1), QTABLES["coarse"], restart=2)[0])
    srcs.append(encode(_smooth_rgb(16, 16, 2), QTABLES["fine"], subsampling=(2, 1), interleaved=False)[0])
    refused = 0
    for it in range(400):
        b = bytearray(srcs[it % len(srcs)])
        if it % 3 == 0:
            b = b[: int(rng.integers(1, len(b)))]
        else:
            for _ in range(int(rng.integers(1, 6))):
                b[int(rng.integers(0, len(b)))] ^= 1 << int(rng.integers(0, 8))
        p = tmp_path / ("f%d" % it)
        p.write_bytes(bytes(b))
        try:
            img = read_hdr(str(p))
        except GbrtError:
            refused += 1
            continue
        assert np.isfinite(img).all() and img.min() >= 0 and img.max() <= 255
    assert refused > 100
