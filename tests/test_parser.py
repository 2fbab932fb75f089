"""The scene-language parser, OBJ/MTL reader and Radiance reader (pure host
code in libgbrt.so; no GPU)."""
import math

import numpy as np
import pytest

from renderer_gb300 import GbrtError, _abi, workloads
from renderer_gb300.scenefile import load_scene, load_scene_string, read_hdr, write_hdr, write_obj, write_scene

pytestmark = pytest.mark.usefixtures("gbrt_built")

CORNELL = """
// A Cornell-style box in the renderer's scene language (colours are RGB).
white = diffuse([0.73 0.73 0.73]);
red = diffuse([0.63 0.065 0.05]);   /* left wall */
green = diffuse([0.14 0.45 0.09]);
intersectable = intersectables {
  quad([-1 0 -1], [1 0 -1], [1 0 1], [-1 0 1], white)
  quad([-1 0 -1], [-1 0 1], [-1 2 1], [-1 2 -1], red)
  quad([1 0 -1], [1 2 -1], [1 2 1], [1 0 1], green)
  sphere([-0.45 0.35 -0.3], 0.35, mirror(1))
  sphere([0.45 0.35 0.25], 0.35, refractive(1.5))
};
lights = lights { arealight([-0.25 1.98 -0.25], [0.5 0 0], [0 0 0.5], [15 15 15]) };
camera = camera([0 1 3.4], [0 1 0], [0 1 0], 0.6981317, 256, 256);
"""


def test_cornell_scene_language():
    s = load_scene_string(CORNELL)
    assert len(s.quads) == 3 and len(s.spheres) == 2 and len(s.lights) == 1
    assert s.camera["width"] == 256 and s.camera["fov"] == pytest.approx(0.6981317)
    red = s.materials[s.quads[1][4]]
    assert red["type"] == _abi.MAT_DIFFUSE
    np.testing.assert_allclose(red["kd"], (0.05, 0.065, 0.63))         # RGB -> BGR
    assert s.materials[s.spheres[0][2]]["type"] == _abi.MAT_MIRROR
    assert s.materials[s.spheres[1][2]]["ior"] == pytest.approx(1.5)
    L = s.lights[0]
    assert L["type"] == _abi.LIGHT_AREA and L["u"] == pytest.approx((0.5, 0, 0))


def test_variables_copy_and_redefinition():
    text = """
    a = diffuse([1 0 0]);
    geo = intersectables { quad([0 0 0], [1 0 0], [1 1 0], [0 1 0], a) };
    a = diffuse([0 1 0]);
    intersectable = geo;
    cam2 = camera([0 0 5], [0 0 0], [0 1 0], 1.0, 32, 16);
    camera = cam2;
    lights = lights { pointlight([0 0 2], [1 2 3]) };
    """
    s = load_scene_string(text)
    # the material seen by the quad is the one defined before its assignment
    np.testing.assert_allclose(s.materials[s.quads[0][4]]["kd"], (0, 0, 1))
    assert s.camera["width"] == 32 and s.camera["height"] == 16
    np.testing.assert_allclose(s.lights[0]["intensity"], (3, 2, 1))


def test_missing_material_is_dark_matter():
    s = load_scene_string("intersectable = intersectables { plane([0 1 0 0], nosuch) };")
    assert s.planes[0][1] == -1


def test_instances_are_flattened():
    text = """
    intersectable = intersectables {
      instance(translate([1 2 3]) * scale(2), intersectables {
        t([0 0 0], [1 0 0], [0 1 0], [0 0 0], [0 0 0], [0 0 0], [0 0], [0 0], [0 0], diffuse([1 1 1]))
        sphere([0 0 0], 0.5, diffuse([1 1 1]))
      })
      instance(rotate(90, [0 0 1]), plane([1 0 0 -1], diffuse([1 1 1])))
    };
    """
    s = load_scene_string(text)
    np.testing.assert_allclose(s.tri_pos[0], [1, 2, 3, 3, 2, 3, 1, 4, 3], atol=1e-6)
    assert s.spheres[0][0] == pytest.approx((1, 2, 3)) and s.spheres[0][1] == pytest.approx(1.0)
    # x = 1 rotated by 90 degrees about z is the plane y = 1
    p = np.array(s.planes[0][0])
    np.testing.assert_allclose(p / np.abs(p).max(), [0, 1, 0, -1], atol=1e-6)


def test_large_instanced_meshes_become_shared_meshes(tmp_path):
    """An obj under instance(...) with at least 1,024 triangles is a shared
    mesh (one per file and material) placed by each instance's transform (a
    two-level BVH); nested transforms multiply; a small one stays
    flattened."""
    pos, _ = workloads.displaced_grid(24, -1, 1, -1, 1, 0, 0.2, 5)   # 1,152 triangles
    write_obj(str(tmp_path / "relief.obj"), pos)
    write_obj(str(tmp_path / "small.obj"), pos[:10])
    text = """
    grey = diffuse([0.5 0.5 0.5]);
    intersectable = intersectables {
      instance(translate([1 0 0]), obj("relief.obj", grey))
      instance(translate([0 2 0]), instance(scale(2), obj("relief.obj", grey)))
      instance(rotate(90, [0 1 0]), obj("small.obj", diffuse([1 1 1])))
    };
    """
    (tmp_path / "s.scene").write_text(text)
    s = load_scene(str(tmp_path / "s.scene"))
    assert len(s.meshes) == 1 and len(s.instances) == 2 and s.n_tri() == 10
    np.testing.assert_allclose(s.meshes[0]["pos"], pos, atol=1e-6)
    t0, t1 = (np.asarray(t) for t, _ in s.instances)
    np.testing.assert_allclose(t0, [[1, 0, 0, 1], [0, 1, 0, 0], [0, 0, 1, 0]], atol=1e-6)
    np.testing.assert_allclose(t1, [[2, 0, 0, 0], [0, 2, 0, 2], [0, 0, 2, 0]], atol=1e-6)
    assert s.prim_offsets()["instances"] == 10


def test_parse_errors_are_reported():
    with pytest.raises(GbrtError) as e:
        load_scene_string("intersectable = intersectables { quad([0 0 0], [1 0 0]) };")
    assert e.value.status == _abi.ERR_PARSE and "line 1" in str(e.value)
    # CSG objects hold at most 8 spheres and boxes
    leaf = "sphere([0 0 0], 1, a)"
    tree = leaf
    for _ in range(8):
        tree = "union(%s, %s)" % (tree, leaf)
    with pytest.raises(GbrtError) as e:
        load_scene_string("x = %s;\nintersectable = x;" % tree)
    assert e.value.status == _abi.ERR_UNSUPPORTED


def test_obj_reader(tmp_path):
    (tmp_path / "m.mtl").write_text("newmtl shiny\nKd 0.5 0.4 0.3\nKs 0.2 0.2 0.2\nNs 40\nillum 2\n"
                                    "newmtl glass\nillum 7\nNi 1.33\n")
    (tmp_path / "m.obj").write_text(
        "mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\n"
        "usemtl shiny\nf 1//1 2//1 3//1 4//1\n"     # a quad face -> a 2-triangle fan
        "usemtl glass\nf -4 -3 -2\n")               # negative (relative) indices
    (tmp_path / "s.scene").write_text('intersectable = intersectables { obj("m.obj", diffuse([1 1 1])) };')
    s = load_scene(str(tmp_path / "s.scene"))
    assert s.n_tri() == 3
    np.testing.assert_allclose(s.tri_pos[1], [0, 0, 0, 1, 1, 0, 0, 1, 0])   # fan (v1, v3, v4)
    m0, m2 = s.materials[s.tri_mat[0]], s.materials[s.tri_mat[2]]
    assert m0["type"] == _abi.MAT_BLINN and m0["exponent"] == 40
    np.testing.assert_allclose(m0["kd"], (0.3, 0.4, 0.5))
    assert m2["type"] == _abi.MAT_TRANSPARENT and m2["ior"] == pytest.approx(1.33)
    np.testing.assert_allclose(s.tri_nrm[0], [0, 0, 1] * 3)


def test_write_then_parse_cornell_roundtrip(tmp_path):
    s = workloads.cornell_box(64, 48)
    p = write_scene(s, str(tmp_path / "cornell.scene"))
    t = load_scene(p)
    assert len(t.quads) == len(s.quads) and len(t.spheres) == len(s.spheres)
    for a, b in zip(s.quads, t.quads):
        np.testing.assert_allclose(np.array(a[:4], float), np.array(b[:4], float))
        np.testing.assert_allclose(s.materials[a[4]]["kd"], t.materials[b[4]]["kd"], rtol=1e-6)
    assert t.camera["width"] == 64 and t.camera["height"] == 48


def test_mesh_roundtrip_through_obj(tmp_path):
    s = workloads.icosphere_scene(levels=2, width=8, height=8, env_size=(16, 8))
    write_hdr(str(tmp_path / "sky.hdr"), s.env)
    p = write_scene(s, str(tmp_path / "ico.scene"), env_file=str(tmp_path / "sky.hdr"))
    t = load_scene(p)
    np.testing.assert_allclose(t.tri_pos, s.tri_pos, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(t.tri_nrm, s.tri_nrm, rtol=1e-5, atol=1e-6)
    assert t.env_mapping == _abi.ENV_LATLONG and t.env.shape == s.env.shape
    # RGBE: one shared exponent, 8 mantissa bits -> error below max(channel) / 128
    assert np.all(np.abs(t.env - s.env) <= s.env.max(-1, keepdims=True) / 128.0 + 1e-30)


def test_rgbe_reader_flat_and_rle(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.uniform(0, 10, (5, 12, 3)).astype(np.float32)
    write_hdr(str(tmp_path / "a.hdr"), img)
    assert np.all(np.abs(read_hdr(str(tmp_path / "a.hdr")) - img) <= img.max(-1, keepdims=True) / 128.0)
    # a run-length encoded file: width 16, every channel a single run
    W, H = 16, 2
    data = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n" % (H, W)
    for _ in range(H):
        data += bytes([2, 2, 0, W])
        for v in (128, 64, 32, 129):          # R G B E
            data += bytes([128 + W, v])
    (tmp_path / "r.hdr").write_bytes(data)
    out = read_hdr(str(tmp_path / "r.hdr"))
    f = 2.0 ** (129 - 136)
    np.testing.assert_allclose(out[0, 0], [32 * f, 64 * f, 128 * f])


def test_reads_the_shipped_angular_probe(reference_probe):
    img = read_hdr(reference_probe)
    assert img.shape == (640, 640, 3) and np.all(np.isfinite(img)) and img.max() > 1.0
    # an angular probe is black outside the unit disc
    assert img[0, 0].max() == 0 and img[320, 320].max() > 0


def test_missing_environment_becomes_black_light():
    s = load_scene_string('lights = lights { environmentmap("does_not_exist.hdr", [1 1 1]) };')
    assert s.lights[0]["type"] == _abi.LIGHT_BLACK and s.env is None


def test_cone_light_parses():
    s = load_scene_string("lights = lights { conelight([0 2 0], [0 -1 0], 0.5, [1 2 3]) };")
    L = s.lights[0]
    assert L["type"] == _abi.LIGHT_CONE and L["u"] == pytest.approx((0, -1, 0)) and L["v"][0] == 0.5
    np.testing.assert_allclose(L["intensity"], (3, 2, 1))
