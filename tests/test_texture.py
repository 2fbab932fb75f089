"""TextureMaterial (src/texturematerial.cpp:33-74): a diffuse material whose
albedo is pow(kd * bilinear(texture, uv), gamma), uv interpolated over
triangles from their texture coordinates (default (0,0), (0,1), (1,0)).

CPU: the oracle against closed forms (a constant texture is a diffuse
material; a textured floor under a point light shows the texel values), the
parser (texture(...) reads PPM, scales by 1/255, unreadable files give
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
