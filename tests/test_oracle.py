"""CPU tests of the oracle (the CPU restatement of the renderer's hot path).

The renderer ships no tests, golden images or scene files and cannot be built
here, so the oracle is pinned against closed-form answers instead: exact ray
parameters of the renderer's intersection formulas, the emission and
next-event formulas of its lights, and whole-image expectations that its
estimator implies analytically (including its quirks).
"""
import math

import numpy as np
import pytest

from oracle.binding import OracleScene, camera_ray, stream_u
from renderer_gb300 import _abi, workloads
from renderer_gb300.runtime import make_rays
from renderer_gb300.scene import SceneData, render_params


def tri_scene(p1, p2, p3, mat_type=_abi.MAT_DIFFUSE):
    s = SceneData()
    s.add_material(mat_type, kd=(0.5, 0.5, 0.5))
    s.tri_pos = np.array([list(p1) + list(p2) + list(p3)], np.float32)
    return s


def test_triangle_hit_distance_and_barycentrics():
    s = tri_scene((0, 0, 0), (1, 0, 0), (0, 1, 0))
    o = OracleScene(s, use_bvh=False)
    h = o.intersect(make_rays([(0.25, 0.25, 5.0)], [(0, 0, -1)]))[0]
    assert h["prim"] == 0 and h["t"] == 5.0
    assert h["u"] == pytest.approx(0.25) and h["v"] == pytest.approx(0.25)
    # Edges are inclusive (u < 0 || u > 1 rejects only outside), misses give NaN.
    h = o.intersect(make_rays([(0.5, 0.5, 1.0), (0.6, 0.6, 1.0)], [(0, 0, -1), (0, 0, -1)]))
    assert h[0]["prim"] == 0 and h[0]["t"] == 1.0
    assert h[1]["prim"] == -1 and math.isnan(h[1]["t"])


def test_ray_range_is_inclusive():
    s = tri_scene((0, 0, 0), (1, 0, 0), (0, 1, 0))
    o = OracleScene(s, use_bvh=False)
    h = o.intersect(make_rays([(0.2, 0.2, 2.0)] * 3, [(0, 0, -1)] * 3, tmin=0.001,
                              tmax=np.array([2.0, 1.999, np.inf], np.float32)))
    assert list(h["prim"]) == [0, -1, 0]


def test_quad_first_triangle_rule_and_single_id():
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(1, 1, 1))
    s.quads = [((-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0), m)]
    o = OracleScene(s)
    rays = make_rays([(-0.5, -0.5, 1), (0.5, 0.5, 1), (0, 0, 1)], [(0, 0, -1)] * 3)
    h = o.intersect(rays)
    assert list(h["prim"]) == [0, 0, 0] and np.all(h["t"] == 1.0)


def test_sphere_csg_rule():
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(1, 1, 1))
    s.spheres = [((0, 0, 0), 1.0, m)]
    o = OracleScene(s)
    h = o.intersect(make_rays([(0, 0, 5), (0, 0, 0), (0, 0, -5)], [(0, 0, -1)] * 3))
    assert h[0]["t"] == 4.0 and h[1]["t"] == 1.0 and math.isnan(h[2]["t"])  # inside: far root


def test_plane_and_environment_hits():
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(1, 1, 1))
    s.planes = [((0, 1, 0, 1.0), m)]      # y = -1
    s.env = np.ones((8, 8, 3), np.float32)
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1))]
    o = OracleScene(s)
    h = o.intersect(make_rays([(0, 0, 0), (0, 0, 0), (0, 0, 0)], [(0, -2, 0), (0, 1, 0), (0, 1, 0)],
                              tmax=np.array([np.inf, np.inf, 10.0], np.float32)))
    assert h[0]["prim"] == 1 and h[0]["t"] == 0.5
    assert h[1]["prim"] == 0 and np.isinf(h[1]["t"])          # the env map at t = +inf
    assert h[2]["prim"] == -1                                   # finite tmax: no env hit


def test_bvh_and_list_agree():
    s = workloads.icosphere_scene(levels=3, width=16, height=16, env_size=(32, 16))
    rng = np.random.default_rng(1)
    org = rng.uniform(-2, 2, (20000, 3))
    d = rng.normal(size=(20000, 3))
    rays = make_rays(org, d)
    a = OracleScene(s, use_bvh=True).intersect(rays, threads=4)
    b = OracleScene(s, use_bvh=False).intersect(rays, threads=4)
    same = a["prim"] == b["prim"]
    assert same.mean() > 0.9999
    np.testing.assert_array_equal(a["t"][same], b["t"][same])


def test_camera_ray_formula():
    cam = _abi.Camera(_abi.F3(0, 1, 3.4), _abi.F3(0, 1, 0), _abi.F3(0, 1, 0), 0.6981317, 256, 256)
    r = camera_ray(cam, 127.5, 127.5)    # the centre of the image: x = y = 0
    np.testing.assert_allclose(r["org"], [0, 1, 3.4], rtol=0, atol=1e-7)
    np.testing.assert_allclose(r["dir"], [0, 0, -1], atol=1e-7)
    r = camera_ray(cam, -0.5, -0.5)      # top-left corner of the image plane
    t = math.tan(0.6981317 / 2)
    np.testing.assert_allclose(r["dir"], [-t, t, -1], rtol=1e-6)


def test_stream_matches_independent_splitmix64():
    M = (1 << 64) - 1

    def mix(z):
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    for seed, sid, dim in [(0, 0, 0), (0, 12345, 7), (99, 1 << 40, 31)]:
        key = mix(seed ^ mix((sid + 0x632BE59BD9B4E019) & M))
        u = (mix((key + dim * 0x9E3779B97F4A7C15) & M) >> 40) / 16777216.0
        assert stream_u(seed, sid, dim) == np.float32(u)


def point_light_plane(width=9, height=9, albedo=0.5, I=4.0):
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(albedo,) * 3)
    s.planes = [((0, 1, 0, 0), m)]                       # y = 0
    s.lights = [dict(type=_abi.LIGHT_POINT, origin=(0, 2, 0), intensity=(I,) * 3)]
    s.camera = dict(eye=(0, 5, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.5, width=width, height=height)
    return s


def test_point_light_next_event_is_closed_form():
    """One diffuse plane lit by a point light, no environment: every sample is
    kd/pi * I / r^2 * cos(theta) (src/pointlight.cpp:29-41, lines 85-98 of the
    integrator); continuation rays leave the scene."""
    s = point_light_plane()
    o = OracleScene(s)
    cam = s.camera_struct()
    r = o.render(cam, render_params(1, 1, 0.5, 5, 0), rng_mode=1)
    # Expected at each pixel sample point: evaluate with the sample's own hit point.
    H, W = cam.height, cam.width
    sid = np.arange(H * W)
    jx = np.array([stream_u(0, int(i), 0) for i in sid]).reshape(H, W)
    jy = np.array([stream_u(0, int(i), 1) for i in sid]).reshape(H, W)
    exp = np.zeros((H, W))
    for y in range(H):
        for x in range(W):
            ray = camera_ray(cam, x + jx[y, x], y + jy[y, x])
            t = -ray["org"][1] / ray["dir"][1]
            p = ray["org"] + t * ray["dir"]
            d = p - np.array([0, 2, 0])
            r2 = d @ d
            cos = abs(d[1]) / math.sqrt(r2)
            exp[y, x] = 0.5 / math.pi * 4.0 / r2 * cos
    np.testing.assert_allclose(r["film"][..., 0], exp, rtol=2e-5)


def test_env_furnace_reference_semantics():
    """A diffuse plane under a constant environment of radiance 1 (reference
    semantics): the continuation ray always reaches the environment, whose
    emission replaces next-event estimation and is weighted by
    brdf * |cos| without the sampling pdf (lines 70-98 of the integrator), so
    the expected pixel value is kd/pi * E[cos] = 2 kd / (3 pi)."""
    s = SceneData()
    kd = 0.6
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(kd,) * 3)
    s.planes = [((0, 1, 0, 0), m)]
    s.env = np.ones((16, 16, 3), np.float32)
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1))]
    s.camera = dict(eye=(0, 5, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.5, width=32, height=32)
    o = OracleScene(s)
    r = o.render(s.camera_struct(), render_params(8, 8, 0.5, 5, 3), rng_mode=0)
    mean = r["film"].mean()
    assert mean == pytest.approx(2 * kd / (3 * math.pi), rel=0.01)


def test_direct_view_of_area_light_uses_unnormalised_camera_direction():
    """A camera ray that hits an area light returns Le * cos * |u x v| / |d|^2 with
    the camera's unnormalised direction d (src/arealight.cpp:53-59, 102-106)."""
    s = SceneData()
    s.lights = [dict(type=_abi.LIGHT_AREA, origin=(-1, -1, 0), u=(2, 0, 0), v=(0, 2, 0),
                     intensity=(3, 3, 3))]      # u x v = (0, 0, 4): faces the camera at +z
    s.camera = dict(eye=(0, 0, 1), look_at=(0, 0, 0), up=(0, 1, 0), fov=0.1, width=3, height=3)
    o = OracleScene(s)
    cam = s.camera_struct()
    r = o.render(cam, render_params(1, 1, 0.5, 5, 0), rng_mode=1)
    for y in range(3):
        for x in range(3):
            sid = y * 3 + x
            ray = camera_ray(cam, x + stream_u(0, sid, 0), y + stream_u(0, sid, 1))
            d = ray["dir"].astype(np.float64)
            cos = -d[2] / np.linalg.norm(d)
            assert r["film"][y, x, 0] == pytest.approx(3 * cos * 4 / (d @ d), rel=1e-5)


def test_path_length_distribution():
    """min(3 + Geometric(p), D) (src/renderer.cpp:52-61) shows up as the ray count
    of a closed scene in which every path reaches its full length: a diffuse
    sphere seen from inside (no light escapes, no emitter is hit)."""
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.5, 0.5, 0.5))
    s.spheres = [((0, 0, 0), 5.0, m)]
    s.lights = [dict(type=_abi.LIGHT_POINT, origin=(0, 0, 0), intensity=(1, 1, 1))]
    s.camera = dict(eye=(0, 0, 0), look_at=(0, 0, -1), up=(0, 1, 0), fov=1.0, width=64, height=64)
    o = OracleScene(s)
    p, D = 0.5, 8
    r = o.render(s.camera_struct(), render_params(2, 2, p, D, 0), rng_mode=1)
    # E[min(3 + K, D)], K ~ Geometric(p) on {0, 1, ...}
    ks = np.arange(0, 64)
    pk = p * (1 - p) ** ks
    exp_len = float(np.sum(np.minimum(3 + ks, D) * pk))
    # The renderer traces pathLength + 1 rays per path (its last intersect is unused).
    assert r["rays"] / r["paths"] == pytest.approx(exp_len + 1, rel=0.01)


def test_cornell_box_reference_render_is_stable():
    s = workloads.cornell_box(32, 32)
    o = OracleScene(s)
    a = o.render(s.camera_struct(), workloads.cornell_params(max_depth=8, seed=5), rng_mode=0, threads=4)
    b = o.render(s.camera_struct(), workloads.cornell_params(max_depth=8, seed=5), rng_mode=0, threads=2)
    np.testing.assert_array_equal(a["film"], b["film"])   # per-row streams: thread-count independent
    assert np.all(np.isfinite(a["film"])) and a["film"].min() >= 0


def test_cone_light_is_a_point_light_inside_its_cone():
    """ConeLight::getIntensity (src/conelight.cpp:31-45): I / r^2 when the angle
    between (x - position) and the axis is within the opening angle, else 0."""
    s = point_light_plane(width=17, height=17)
    s.lights = [dict(type=_abi.LIGHT_CONE, origin=(0, 2, 0), u=(0, -1, 0), v=(0.3, 0, 0), intensity=(4.0,) * 3)]
    o = OracleScene(s)
    cam = s.camera_struct()
    r = o.render(cam, render_params(1, 1, 0.5, 5, 0), rng_mode=1)
    f = r["film"][..., 0]
    ref = OracleScene(point_light_plane(width=17, height=17)).render(cam, render_params(1, 1, 0.5, 5, 0),
                                                                      rng_mode=1)["film"][..., 0]
    inside = f > 0
    assert 0 < inside.sum() < f.size                       # the cone cuts the lit disc
    np.testing.assert_array_equal(f[inside], ref[inside])  # inside it is exactly the point light


# ------------------------------------------------------- physical semantics
def phys(x=8, y=8, D=8, seed=0, p=0.5):
    return render_params(x, y, p, D, seed, semantics=_abi.SEM_PHYSICAL)


def lambert_irradiance(x, n, verts, Le):
    """Irradiance at x (normal n) from a uniform polygonal emitter (Lambert)."""
    E = 0.0
    v = [(np.asarray(p, float) - x) / np.linalg.norm(np.asarray(p, float) - x) for p in verts]
    for i in range(len(v)):
        a, b = v[i], v[(i + 1) % len(v)]
        c = np.cross(a, b)
        E += math.acos(np.clip(a @ b, -1, 1)) * (n @ c) / np.linalg.norm(c)
    return abs(E) * Le / 2


def area_light_scene(kd=0.5, Le=3.0, width=4, fov=0.02):
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(kd,) * 3)
    s.planes = [((0, 1, 0, 0), m)]
    s.lights = [dict(type=_abi.LIGHT_AREA, origin=(-0.5, 1, -0.5), u=(1, 0, 0), v=(0, 0, 1), intensity=(Le,) * 3)]
    s.camera = dict(eye=(0, 0.5, 3), look_at=(0.2, 0, 0.1), up=(0, 1, 0), fov=fov, width=width, height=width)
    return s


def test_physical_furnace():
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.6,) * 3)
    s.planes = [((0, 1, 0, 0), m)]
    s.env = np.ones((16, 16, 3), np.float32)
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1))]
    s.camera = dict(eye=(0, 5, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.5, width=32, height=32)
    r = OracleScene(s).render(s.camera_struct(), phys(8, 8, 8, 3), rng_mode=0)
    assert r["film"].mean() == pytest.approx(0.6, rel=0.01)


def test_physical_area_light_matches_lambert_formula():
    s = area_light_scene()
    r = OracleScene(s).render(s.camera_struct(), phys(32, 32, 4, 1), rng_mode=0)
    assert r["film"].mean() == pytest.approx(footprint_lambert(s), rel=0.01)


def footprint_lambert(s, kd=0.5, Le=3.0, per_pixel=10):
    """Image mean of the area-light scene: kd/pi * E averaged over the points
    of the floor the camera's rays reach (the view is grazing, so a pixel
    covers a strip of the floor over which E changes by several percent)."""
    from oracle.binding import camera_ray
    cam = s.camera_struct()
    verts = [(-0.5, 1, -0.5), (0.5, 1, -0.5), (0.5, 1, 0.5), (-0.5, 1, 0.5)]
    w = s.camera["width"]
    grid = (np.arange(w * per_pixel) + 0.5) / per_pixel
    vals = []
    for py in grid:
        for px in grid:
            ray = camera_ray(cam, px, py)
            o, d = np.array(ray["org"], float), np.array(ray["dir"], float)
            vals.append(lambert_irradiance(o - o[1] / d[1] * d, np.array([0, 1.0, 0]), verts, Le))
    return kd / math.pi * float(np.mean(vals))


def test_physical_direct_view_of_area_light_is_Le():
    s = SceneData()
    s.lights = [dict(type=_abi.LIGHT_AREA, origin=(-1, -1, 0), u=(2, 0, 0), v=(0, 2, 0), intensity=(3, 2, 1))]
    s.camera = dict(eye=(0, 0, 1), look_at=(0, 0, 0), up=(0, 1, 0), fov=0.1, width=3, height=3)
    r = OracleScene(s).render(s.camera_struct(), phys(1, 1), rng_mode=1)
    np.testing.assert_allclose(r["film"].reshape(-1, 3), np.tile([3, 2, 1], (9, 1)), rtol=1e-6)
