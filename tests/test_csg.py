"""CSG objects (src/csgobject.cpp:25-44, src/csgoperation.cpp:27-97,
src/sphere.cpp:29-56, src/axisalignedbox.cpp:30-73): interval lists of
spheres and boxes merged by intersection, union, difference and xor; a hit is
the first boundary at or beyond the ray's start.

CPU: the oracle against closed forms (including the box's exit boundary that
keeps the entry face's normal) and the parser (box and CSG trees become CSG
objects). GPU: ray-level parity of the traversal with the oracle (same
primitive, bit-identical t) and path-level parity of a render."""
import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import _abi
from renderer_gb300.runtime import make_rays
from renderer_gb300.scene import SceneData, render_params


def csg_scene():
    s = SceneData()
    red = s.add_material(_abi.MAT_DIFFUSE, kd=(0.1, 0.1, 0.7))
    white = s.add_material(_abi.MAT_DIFFUSE, kd=(0.7, 0.7, 0.7))
    glass = s.add_material(_abi.MAT_TRANSPARENT, ior=1.5)
    # a box with a spherical bite (diff), two overlapping spheres (isect),
    # a lens of two spheres (xor), a union of a box and a sphere, a lone box;
    # boxes float just above the floor (a face on the plane would tie with it)
    b = s.csg_leaf(_abi.CSG_BOX, (-1, 0.02, -1), (0, 1, 0), red)
    bite = s.csg_leaf(_abi.CSG_SPHERE, (0, 1, 0), (0.6, 0, 0), white)
    s.add_csg(s.csg_op(_abi.CSG_DIFF, b, bite))
    s1 = s.csg_leaf(_abi.CSG_SPHERE, (1.0, 0.5, 0), (0.5, 0, 0), glass)
    s2 = s.csg_leaf(_abi.CSG_SPHERE, (1.4, 0.5, 0), (0.5, 0, 0), white)
    s.add_csg(s.csg_op(_abi.CSG_ISECT, s1, s2))
    s3 = s.csg_leaf(_abi.CSG_SPHERE, (0, 0.5, 1.5), (0.4, 0, 0), red)
    s4 = s.csg_leaf(_abi.CSG_SPHERE, (0.3, 0.5, 1.5), (0.4, 0, 0), white)
    s.add_csg(s.csg_op(_abi.CSG_XOR, s3, s4))
    b2 = s.csg_leaf(_abi.CSG_BOX, (1.2, 0.03, 1.2), (1.8, 0.4, 1.8), white)
    s5 = s.csg_leaf(_abi.CSG_SPHERE, (1.5, 0.5, 1.5), (0.25, 0, 0), red)
    s.add_csg(s.csg_op(_abi.CSG_UNION, b2, s5))
    s.add_csg(s.csg_leaf(_abi.CSG_BOX, (-1.8, 0.01, 1.0), (-1.2, 0.8, 1.6), white))
    s.planes = [((0, 1, 0, 0), white)]
    s.lights = [dict(type=_abi.LIGHT_AREA, origin=(-0.5, 3, -0.5), u=(1, 0, 0), v=(0, 0, 1), intensity=(8, 8, 8)),
                dict(type=_abi.LIGHT_POINT, origin=(2, 3, 3), intensity=(6, 6, 6))]
    s.camera = dict(eye=(0.5, 2.5, 5), look_at=(0.2, 0.4, 0.3), up=(0, 1, 0), fov=0.7, width=64, height=48)
    return s


def one(s, o, d, tmin=0.001):
    h = OracleScene(s).intersect(make_rays(np.array([o], np.float32), np.array([d], np.float32), tmin=tmin),
                                 threads=1)
    return h[0]


def test_box_entry_and_exit():
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.5, 0.5, 0.5))
    s.add_csg(s.csg_leaf(_abi.CSG_BOX, (-1, -1, -1), (1, 1, 1), m))
    s.camera = dict(eye=(0, 0, 5), look_at=(0, 0, 0), up=(0, 1, 0), fov=0.5, width=4, height=4)
    assert one(s, (0, 0, 5), (0, 0, -1))["t"] == pytest.approx(4.0)
    assert one(s, (0, 0, 0), (0, 0, -1))["t"] == pytest.approx(1.0)  # from inside: the exit
    assert np.isnan(one(s, (3, 0, 5), (0, 0, -1))["t"])


def test_operations_closed_forms():
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.5, 0.5, 0.5))
    a = s.csg_leaf(_abi.CSG_SPHERE, (0, 0, 0), (1, 0, 0), m)
    b = s.csg_leaf(_abi.CSG_SPHERE, (1, 0, 0), (1, 0, 0), m)
    s.add_csg(s.csg_op(_abi.CSG_DIFF, a, b))
    s.camera = dict(eye=(0, 0, 5), look_at=(0, 0, 0), up=(0, 1, 0), fov=0.5, width=4, height=4)
    # along +x from -5: enter a at x = -1
    assert one(s, (-5, 0, 0), (1, 0, 0))["t"] == pytest.approx(4.0)
    # along -x from +5: b covers a on this side; the bite's wall is b's entry at x = 0
    assert one(s, (5, 0, 0), (-1, 0, 0))["t"] == pytest.approx(5.0)
    for op, t in ((_abi.CSG_ISECT, 4.0), (_abi.CSG_UNION, 3.0), (_abi.CSG_XOR, 3.0)):
        s.csg_nodes[-1] = (op, a, b, (0, 0, 0), (0, 0, 0), -1)
        assert one(s, (5, 0, 0), (-1, 0, 0))["t"] == pytest.approx(t), op


def test_parser_builds_csg_objects():
    from renderer_gb300.scenefile import load_scene_string
    s = load_scene_string("m = diffuse([0.5 0.5 0.5]);\nintersectable = intersectables { box([0 0 0], [1 1 1], m) "
                          "diff(box([2 0 0], [3 1 1], m), sphere([2.5 1 0.5], 0.3, m)) "
                          "instance(translate([2 0 0]), box([0 0 0], [1 1 1], m)) };")
    assert len(s.quads) == 0 and len(s.csg_roots) == 3
    ops = [n[0] for n in s.csg_nodes]
    assert ops.count(_abi.CSG_BOX) == 3 and ops.count(_abi.CSG_DIFF) == 1 and ops.count(_abi.CSG_SPHERE) == 1
    moved = s.csg_nodes[s.csg_roots[2]]
    assert moved[3] == pytest.approx((2, 0, 0)) and moved[4] == pytest.approx((3, 1, 1))


@pytest.mark.gpu
def test_csg_ray_parity(ctx):
    from renderer_gb300.runtime import GpuScene
    from tests.test_gpu_trace import box_rays, compare
    rng = np.random.default_rng(4)
    s = csg_scene()
    gs = GpuScene(ctx, s)
    orc = OracleScene(s)
    rays = box_rays(s, rng, 200000)
    compare(gs.intersect(rays), orc.intersect(rays, threads=0), "csg")
    inside = make_rays(rng.uniform(-0.9, -0.1, (5000, 3)) * [1, -1, 1] + [0, 0, 0],
                       rng.normal(size=(5000, 3)))
    compare(gs.intersect(inside), orc.intersect(inside, threads=0), "csg-inside")


@pytest.mark.gpu
@pytest.mark.parametrize("semantics", [_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL])
def test_csg_path_level_parity(ctx, semantics):
    from tests.test_gpu_render import gpu_render
    s = csg_scene()
    prm = render_params(2, 2, 0.5, 6, 5, semantics=semantics)
    (film, _, _), _ = gpu_render(ctx, s, prm)
    orc = OracleScene(s).render(s.camera_struct(), prm, rng_mode=1)["film"]
    close = np.isclose(film, orc, rtol=2e-3, atol=1e-5).all(-1)
    assert close.mean() > 0.97, close.mean()
    assert film.mean() == pytest.approx(orc.mean(), rel=5e-3)
