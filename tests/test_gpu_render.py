"""Image-level parity of the CUDA path tracer with the oracle's
PerPixelRenderer + UniDiPathTracingIntegrator (reference semantics).

Three kinds of check:
  * closed forms that the renderer's estimator implies (point-light next-event
    estimation, the environment "furnace", direct view of an area light);
  * path-level parity: with the counter-based stream both sides draw the same
    numbers for every camera sample, so per-pixel results agree up to float
    rounding (rare discrete flips are allowed as a small fraction of pixels);
  * statistical parity with independent streams: per-pixel z-test on mean and
    variance, with a binomial bound on the count of |z| > 4.
"""
import math

import numpy as np
import pytest
from scipy import stats as sst

from oracle.binding import OracleScene, camera_ray, stream_u
from renderer_gb300 import GpuScene, PerPixelRenderer, _abi, workloads
from renderer_gb300.scene import SceneData, render_params

pytestmark = pytest.mark.gpu


def gpu_render(ctx, s, params, moments=True):
    gs = GpuScene(ctx, s)
    r = PerPixelRenderer(gs, s.camera_struct())
    r.params = params
    out = r.render(want_moments=moments)
    return out, r.stats


def test_point_light_closed_form(ctx):
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.5,) * 3)
    s.planes = [((0, 1, 0, 0), m)]
    s.lights = [dict(type=_abi.LIGHT_POINT, origin=(0, 2, 0), intensity=(4.0,) * 3)]
    s.camera = dict(eye=(0, 5, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.5, width=9, height=9)
    (film, _, _), st = gpu_render(ctx, s, render_params(1, 1, 0.5, 5, 0))
    cam = s.camera_struct()
    exp = np.zeros((9, 9))
    for y in range(9):
        for x in range(9):
            sid = y * 9 + x
            ray = camera_ray(cam, x + stream_u(0, sid, 0), y + stream_u(0, sid, 1))
            t = -ray["org"][1] / ray["dir"][1]
            p = ray["org"] + t * ray["dir"]
            d = p - np.array([0, 2, 0])
            exp[y, x] = 0.5 / math.pi * 4.0 / (d @ d) * abs(d[1]) / math.sqrt(d @ d)
    np.testing.assert_allclose(film[..., 0], exp, rtol=1e-4)
    assert st.paths == 81 and st.nonfinite == 0


def test_cone_light_closed_form(ctx):
    """A cone light on a diffuse plane: inside the cone the sample is the
    point-light value (same per-sample random numbers as the oracle)."""
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.5,) * 3)
    s.planes = [((0, 1, 0, 0), m)]
    s.lights = [dict(type=_abi.LIGHT_CONE, origin=(0, 2, 0), u=(0, -1, 0), v=(0.3, 0, 0), intensity=(4.0,) * 3)]
    s.camera = dict(eye=(0, 5, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.5, width=17, height=17)
    params = render_params(1, 1, 0.5, 5, 0)
    (film, _, _), _ = gpu_render(ctx, s, params)
    ref = OracleScene(s).render(s.camera_struct(), params, rng_mode=1)["film"]
    inside = ref[..., 0] > 0
    assert 0 < inside.sum() < inside.size
    np.testing.assert_allclose(film, ref, rtol=1e-4, atol=1e-7)


def test_env_furnace(ctx):
    s = SceneData()
    kd = 0.6
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(kd,) * 3)
    s.planes = [((0, 1, 0, 0), m)]
    s.env = np.ones((16, 16, 3), np.float32)
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1))]
    s.camera = dict(eye=(0, 5, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.5, width=64, height=64)
    (film, _, _), _ = gpu_render(ctx, s, render_params(8, 8, 0.5, 5, 11))
    assert film.mean() == pytest.approx(2 * kd / (3 * math.pi), rel=0.005)


def test_direct_view_of_area_light(ctx):
    s = SceneData()
    s.lights = [dict(type=_abi.LIGHT_AREA, origin=(-1, -1, 0), u=(2, 0, 0), v=(0, 2, 0), intensity=(3, 3, 3))]
    s.camera = dict(eye=(0, 0, 1), look_at=(0, 0, 0), up=(0, 1, 0), fov=0.1, width=3, height=3)
    (film, _, _), _ = gpu_render(ctx, s, render_params(1, 1, 0.5, 5, 0))
    cam = s.camera_struct()
    for y in range(3):
        for x in range(3):
            sid = y * 3 + x
            d = camera_ray(cam, x + stream_u(0, sid, 0), y + stream_u(0, sid, 1))["dir"].astype(np.float64)
            assert film[y, x, 0] == pytest.approx(3 * (-d[2] / np.linalg.norm(d)) * 4 / (d @ d), rel=1e-5)


def path_level(ctx, s, params, rel=2e-3, min_frac=0.98):
    (film, _, _), st = gpu_render(ctx, s, params)
    o = OracleScene(s).render(s.camera_struct(), params, rng_mode=1)
    a, b = film.astype(np.float64), o["film"].astype(np.float64)
    close = np.abs(a - b) <= rel * np.maximum(np.abs(b), 1e-3)
    frac = close.all(-1).mean()
    assert frac >= min_frac, frac
    # global energy agrees tightly even with a few flipped paths
    assert a.sum() == pytest.approx(b.sum(), rel=5e-3)
    assert st.nonfinite == 0
    return frac, st, o


def test_path_level_parity_cornell(ctx):
    s = workloads.cornell_box(64, 64)
    frac, st, o = path_level(ctx, s, workloads.cornell_params(max_depth=8, seed=7))
    assert st.paths == 64 * 64 * 16
    # one extension ray fewer per path than the oracle: the renderer's last
    # intersect of a full-length path is never used and is not traced here
    assert st.extension_rays <= o["rays"]


def test_path_level_parity_cornell_depth5(ctx):
    s = workloads.cornell_box(48, 48)
    path_level(ctx, s, workloads.cornell_params(max_depth=5, seed=3))


def test_path_level_parity_icosphere(ctx):
    s = workloads.icosphere_scene(levels=4, width=48, height=48, env_size=(128, 64))
    path_level(ctx, s, render_params(4, 4, 0.5, 12, 5))


def test_path_level_parity_materials(ctx):
    """Blinn, Phong, mirror and glass spheres on a diffuse floor under an
    angular light probe plus a point light and an area light."""
    s = SceneData()
    floor = s.add_material(_abi.MAT_DIFFUSE, kd=(0.4, 0.5, 0.6))
    blinn = s.add_material(_abi.MAT_BLINN, kd=(0.3, 0.2, 0.1), ks=(0.4, 0.4, 0.4), exponent=60)
    phong = s.add_material(_abi.MAT_PHONG, kd=(0.2, 0.5, 0.2), ks=(0.3, 0.3, 0.3), exponent=20)
    mirror = s.add_material(_abi.MAT_MIRROR)
    glass = s.add_material(_abi.MAT_TRANSPARENT, ior=1.5)
    s.planes = [((0, 1, 0, 0), floor)]
    s.spheres = [((-1.5, 0.5, 0), 0.5, blinn), ((-0.5, 0.5, 0), 0.5, phong), ((0.5, 0.5, 0), 0.5, mirror),
                 ((1.5, 0.5, 0), 0.5, glass)]
    rng = np.random.default_rng(4)
    s.env = rng.uniform(0.2, 1.0, (32, 32, 3)).astype(np.float32)
    s.env_mapping = _abi.ENV_ANGULAR
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1)),
                dict(type=_abi.LIGHT_POINT, origin=(0, 3, 2), intensity=(5, 5, 5)),
                dict(type=_abi.LIGHT_AREA, origin=(-1, 3, -1), u=(2, 0, 0), v=(0, 0, 2), intensity=(4, 4, 4))]
    s.camera = dict(eye=(0, 1.5, 5), look_at=(0, 0.5, 0), up=(0, 1, 0), fov=0.8, width=64, height=48)
    path_level(ctx, s, render_params(4, 4, 0.5, 8, 9), min_frac=0.97)


def test_statistical_parity_cornell(ctx):
    """Independent streams (oracle: per-row Tausworthe; GPU: counter-based)."""
    s = workloads.cornell_box(64, 64)
    params = workloads.cornell_params(max_depth=8, seed=1, x_samples=8, y_samples=8)
    (film, gs, gq), _ = gpu_render(ctx, s, params)
    o = OracleScene(s).render(s.camera_struct(), params, rng_mode=0)
    N = 64
    ma, mb = gs / N, o["sum"] / N
    va = np.maximum(gq / N - ma ** 2, 0) * N / (N - 1)
    vb = np.maximum(o["sumsq"] / N - mb ** 2, 0) * N / (N - 1)
    se = np.sqrt(va / N + vb / N)
    ok = se > 0
    z = (ma - mb)[ok] / se[ok]
    m = z.size
    # expected count of |z| > 4 under the null is tiny; allow the binomial 1e-6 upper quantile
    p4 = 2 * sst.norm.sf(4.0)
    bound = sst.binom.ppf(1 - 1e-6, m, p4) + 5   # +5: heavy-tailed caustic pixels
    assert (np.abs(z) > 4).sum() <= bound
    assert abs(z.mean()) < 0.05
    rel_mean = abs(ma.mean() - mb.mean()) / mb.mean()
    assert rel_mean < 0.01


def test_cancellation_flag(ctx):
    import ctypes
    s = workloads.cornell_box(32, 32)
    gs = GpuScene(ctx, s)
    r = PerPixelRenderer(gs, s.camera_struct())
    flag = ctypes.c_int32(1)
    from renderer_gb300 import GbrtError
    with pytest.raises(GbrtError) as e:
        r.render(stop_flag=flag)
    assert e.value.status == _abi.ERR_CANCELLED


def test_gpu_tonemap_matches_oracle(ctx):
    import ctypes

    import torch

    import renderer_gb300 as rg
    from oracle.binding import tonemap as oracle_tonemap
    rng = np.random.default_rng(2)
    f = rng.uniform(0, 2, (123, 77, 3)).astype(np.float32)
    f[0, 0] = (np.nan, -3, 1e9)
    d = torch.from_numpy(f).cuda()
    o = torch.zeros(f.shape, dtype=torch.uint8, device="cuda")
    rg.check(rg.lib().gbrt_tonemap_device(ctx.handle, ctypes.c_void_p(d.data_ptr()), 77, 123, 2.2,
                                          ctypes.c_void_p(o.data_ptr()), None))
    torch.cuda.synchronize()
    got = o.cpu().numpy()
    ref = oracle_tonemap(f, 2.2)
    diff = np.abs(got.astype(int) - ref.astype(int))
    assert diff.max() <= 1 and (diff > 0).mean() < 1e-4   # pow(double) rounding at integer boundaries


# ------------------------------------------------------- physical semantics
def phys(x=8, y=8, D=8, seed=0, p=0.5):
    return render_params(x, y, p, D, seed, semantics=_abi.SEM_PHYSICAL)


def test_physical_closed_forms(ctx):
    from tests.test_oracle import area_light_scene, footprint_lambert
    s = area_light_scene()
    (film, _, _), st = gpu_render(ctx, s, phys(32, 32, 4, 1))
    assert film.mean() == pytest.approx(footprint_lambert(s), rel=0.01)
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.6,) * 3)
    s.planes = [((0, 1, 0, 0), m)]
    s.env = np.ones((16, 16, 3), np.float32)
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1))]
    s.camera = dict(eye=(0, 5, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.5, width=64, height=64)
    (film, _, _), _ = gpu_render(ctx, s, phys(8, 8, 8, 5))
    assert film.mean() == pytest.approx(0.6, rel=0.005)


def test_physical_path_level_parity(ctx):
    s = workloads.cornell_box(48, 48)
    path_level(ctx, s, phys(4, 4, 8, 2), min_frac=0.97)


def test_physical_path_level_parity_materials(ctx):
    s = SceneData()
    floor = s.add_material(_abi.MAT_DIFFUSE, kd=(0.4, 0.5, 0.6))
    blinn = s.add_material(_abi.MAT_BLINN, kd=(0.3, 0.2, 0.1), ks=(0.4, 0.4, 0.4), exponent=60)
    phong = s.add_material(_abi.MAT_PHONG, kd=(0.2, 0.5, 0.2), ks=(0.3, 0.3, 0.3), exponent=20)
    mirror = s.add_material(_abi.MAT_MIRROR)
    glass = s.add_material(_abi.MAT_TRANSPARENT, ior=1.5)
    s.planes = [((0, 1, 0, 0), floor)]
    s.spheres = [((-1.5, 0.5, 0), 0.5, blinn), ((-0.5, 0.5, 0), 0.5, phong), ((0.5, 0.5, 0), 0.5, mirror),
                 ((1.5, 0.5, 0), 0.5, glass)]
    rng = np.random.default_rng(4)
    s.env = rng.uniform(0.2, 1.0, (32, 32, 3)).astype(np.float32)
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1)),
                dict(type=_abi.LIGHT_POINT, origin=(0, 3, 2), intensity=(5, 5, 5)),
                dict(type=_abi.LIGHT_AREA, origin=(-1, 3, -1), u=(2, 0, 0), v=(0, 0, 2), intensity=(4, 4, 4))]
    s.camera = dict(eye=(0, 1.5, 5), look_at=(0, 0.5, 0), up=(0, 1, 0), fov=0.8, width=64, height=48)
    path_level(ctx, s, phys(4, 4, 8, 9), min_frac=0.97)


def test_physical_statistical_parity(ctx):
    s = workloads.cornell_box(48, 48)
    params = phys(8, 8, 8, 3)
    (film, gs, gq), _ = gpu_render(ctx, s, params)
    o = OracleScene(s).render(s.camera_struct(), params, rng_mode=0)
    N = 64
    ma, mb = gs / N, o["sum"] / N
    va = np.maximum(gq / N - ma ** 2, 0) * N / (N - 1)
    vb = np.maximum(o["sumsq"] / N - mb ** 2, 0) * N / (N - 1)
    se = np.sqrt(va / N + vb / N)
    ok = se > 0
    z = (ma - mb)[ok] / se[ok]
    bound = sst.binom.ppf(1 - 1e-6, z.size, 2 * sst.norm.sf(4.0)) + 5
    assert (np.abs(z) > 4).sum() <= bound
    assert abs(z.mean()) < 0.05
    assert abs(ma.mean() - mb.mean()) / mb.mean() < 0.01


@pytest.mark.gpu
def test_context_pool_keeps_then_trims(ctx):
    """Renders reuse the context pool's memory; trimming hands it back."""
    s = workloads.cornell_box(64, 64)
    r = PerPixelRenderer(GpuScene(ctx, s), options={"pt-x-samples": 2, "pt-y-samples": 2})
    a = r.render()
    b = r.render()
    assert np.allclose(a, b, rtol=1e-6, atol=1e-7)  # same paths; shadow-ray adds are atomics
    assert ctx.trim() == 0
