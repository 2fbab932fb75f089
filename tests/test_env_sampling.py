"""Importance sampling of the environment map by the physical estimator (not
part of the renderer, whose next-event estimation draws the cosine,
src/environmentmap.cpp:40-54): the oracle and the GPU against a closed form,
against each other path by path, and against uniform sampling
(GBRT_SCENE_ENV_UNIFORM) for variance.

The closed form: a diffuse plane under a lat-long map that is constant per
texel is lit by E = sum over the upper rows of L_texel * (pi / W) *
(sin^2 theta_1 - sin^2 theta_0); every point of the plane shows kd / pi * E.
"""
import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import _abi
from renderer_gb300.scene import SceneData, render_params

KD = 0.6


def sun_sky(W=64, H=32, sun=(8, 20), sun_radiance=2000.0):
    """A gradient sky (BGR) with one bright texel."""
    v = (np.arange(H) + 0.5) / H
    sky = np.zeros((H, W, 3), np.float32)
    sky[..., 0] = (0.3 + 0.7 * (1 - v))[:, None]   # blue, brighter at the zenith
    sky[..., 1] = 0.4
    sky[..., 2] = 0.2 + 0.1 * np.cos(np.linspace(0, 2 * np.pi, W))[None, :]
    sky[sun[0], sun[1]] = sun_radiance
    return sky


def plane_scene(sky, flags=0, mapping=_abi.ENV_LATLONG, size=24):
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(KD,) * 3)
    s.planes = [((0, 1, 0, 0), m)]
    s.env = sky
    s.env_mapping = mapping
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1))]
    s.camera = dict(eye=(0, 5, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.4, width=size, height=size)
    s.flags = flags
    return s


def irradiance(sky):
    H, W, _ = sky.shape
    th0 = np.pi * np.arange(H) / H
    th1 = np.pi * (np.arange(H) + 1) / H
    wgt = np.where(np.arange(H) < H // 2, (np.pi / W) * (np.sin(th1) ** 2 - np.sin(th0) ** 2), 0.0)
    return (sky.astype(np.float64) * wgt[:, None, None]).sum((0, 1))


def phys(xs, seed, D=4):
    return render_params(xs, xs, 0.5, D, seed, semantics=_abi.SEM_PHYSICAL)


# ------------------------------------------------------------------- CPU ----
def test_oracle_importance_sampling_converges_to_the_closed_form():
    sky = sun_sky()
    want = KD / np.pi * irradiance(sky)
    s = plane_scene(sky)
    o = OracleScene(s).render(s.camera_struct(), phys(16, 3), rng_mode=1)
    got = o["film"].reshape(-1, 3).mean(0)
    np.testing.assert_allclose(got, want, rtol=0.01)


def test_oracle_importance_sampling_beats_uniform_on_a_sun():
    sky = sun_sky()
    want = KD / np.pi * irradiance(sky)
    errs = []
    for flags in (0, _abi.SCENE_ENV_UNIFORM):
        s = plane_scene(sky, flags)
        o = OracleScene(s).render(s.camera_struct(), phys(4, 9), rng_mode=1)
        errs.append(float(np.mean((o["film"].astype(np.float64) - want) ** 2)))
    # uniform sampling finds the one-texel sun by chance; importance sampling
    # draws it in proportion to its share of the irradiance
    assert errs[0] * 20 < errs[1], errs


def test_oracle_angular_importance_sampling_is_unbiased():
    """An angular probe (the renderer's mapping, +x at the disc's centre) with
    a sun in the plane's upper hemisphere (cx > 0): importance-sampled and
    uniform next-event estimation converge to the same image."""
    sky = sun_sky(48, 48, sun=(30, 36), sun_radiance=100.0)
    means = []
    for flags in (0, _abi.SCENE_ENV_UNIFORM):
        s = plane_scene(sky, flags, _abi.ENV_ANGULAR)
        o = OracleScene(s).render(s.camera_struct(), phys(24 if flags == 0 else 128, 4), rng_mode=1)
        means.append(o["film"].reshape(-1, 3).astype(np.float64).mean(0))
    np.testing.assert_allclose(means[0], means[1], rtol=0.01)


# ------------------------------------------------------------------- GPU ----
@pytest.mark.gpu
@pytest.mark.parametrize("flags", [0, _abi.SCENE_ENV_UNIFORM])
def test_gpu_environment_closed_form(ctx, flags):
    from renderer_gb300 import GpuScene, PerPixelRenderer
    sky = sun_sky()
    want = KD / np.pi * irradiance(sky)
    s = plane_scene(sky, flags, size=32)
    r = PerPixelRenderer(GpuScene(ctx, s), s.camera_struct())
    r.params = phys(64 if flags == 0 else 128, 5)
    film = r.render()
    np.testing.assert_allclose(film.reshape(-1, 3).mean(0), want, rtol=0.005 if flags == 0 else 0.02)
    assert r.stats.nonfinite == 0


@pytest.mark.gpu
@pytest.mark.parametrize("mapping", [_abi.ENV_LATLONG, _abi.ENV_ANGULAR])
def test_gpu_environment_sampling_path_level(ctx, mapping):
    """The same random numbers on both sides: the same sampled directions,
    the same densities and MIS weights."""
    from renderer_gb300 import GpuScene, PerPixelRenderer
    rng = np.random.default_rng(6)
    # the sun above the plane in either mapping
    sun = (12, 30) if mapping == _abi.ENV_LATLONG else (30, 36)
    sky = sun_sky(48, 48, sun=sun, sun_radiance=500.0) * rng.uniform(0.5, 1.5, (48, 48, 1)).astype(np.float32)
    s = plane_scene(sky, 0, mapping, size=32)
    glossy = s.add_material(_abi.MAT_BLINN, kd=(0.2, 0.3, 0.4), ks=(0.5, 0.5, 0.5), exponent=40)
    s.spheres = [((0.3, 0.4, 0.2), 0.4, glossy)]
    params = phys(4, 8, D=6)
    r = PerPixelRenderer(GpuScene(ctx, s), s.camera_struct())
    r.params = params
    film = r.render().astype(np.float64)
    ref = OracleScene(s).render(s.camera_struct(), params, rng_mode=1)["film"].astype(np.float64)
    close = (np.abs(film - ref) <= 2e-3 * np.maximum(np.abs(ref), 1e-3)).all(-1)
    assert close.mean() >= 0.97, close.mean()
    assert film.sum() == pytest.approx(ref.sum(), rel=5e-3)


@pytest.mark.gpu
def test_gpu_importance_sampling_lowers_the_error(ctx):
    from renderer_gb300 import GpuScene, PerPixelRenderer
    sky = sun_sky()
    want = KD / np.pi * irradiance(sky)
    err = []
    for flags in (0, _abi.SCENE_ENV_UNIFORM):
        s = plane_scene(sky, flags, size=64)
        r = PerPixelRenderer(GpuScene(ctx, s), s.camera_struct())
        r.params = phys(2, 13)
        err.append(float(np.mean((r.render().astype(np.float64) - want) ** 2)))
    assert err[0] * 20 < err[1], err
