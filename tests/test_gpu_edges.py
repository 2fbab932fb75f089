"""Edge cases of the render call, path by path against the oracle: a 1x1
image, ragged wavefronts (batch_paths that divide neither the image nor the
sample count), the shortest paths (max depth 1), a scene without lights,
and a scene without geometry (only the environment map), in both estimators.
"""
import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import GpuScene, PerPixelRenderer, _abi, workloads
from renderer_gb300.scene import SceneData, render_params

pytestmark = pytest.mark.gpu


def render_both(ctx, s, params):
    r = PerPixelRenderer(GpuScene(ctx, s), s.camera_struct())
    r.params = params
    film, _, _ = r.render(want_moments=True)
    o = OracleScene(s).render(s.camera_struct(), params, rng_mode=1)
    return film.astype(np.float64), o["film"].astype(np.float64), r.stats, o


def assert_path_level(a, b, rel=2e-3, min_frac=0.98):
    close = np.abs(a - b) <= rel * np.maximum(np.abs(b), 1e-3)
    assert close.all(-1).mean() >= min_frac
    assert a.sum() == pytest.approx(b.sum(), rel=5e-3, abs=1e-9)


@pytest.mark.parametrize("semantics", [_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL])
def test_single_pixel_single_sample(ctx, semantics):
    s = workloads.cornell_box(1, 1)
    p = render_params(1, 1, 0.5, 8, 3, semantics=semantics)
    a, b, st, o = render_both(ctx, s, p)
    assert a.shape == (1, 1, 3) and st.paths == 1 == o["paths"]
    np.testing.assert_allclose(a, b, rtol=2e-3, atol=1e-6)


@pytest.mark.parametrize("semantics", [_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL])
def test_ragged_wavefronts(ctx, semantics):
    """37 x 19 pixels at 3 x 1 spp (2,109 paths) in wavefronts of 1,000: the
    last wavefront holds 109 paths and splits a pixel's samples across
    wavefronts; the image equals the one-wavefront render and the oracle's."""
    s = workloads.cornell_box(37, 19)
    p = render_params(3, 1, 0.5, 8, 11, semantics=semantics)
    a, b, st, _ = render_both(ctx, s, p)
    p.batch_paths = 1000
    r = PerPixelRenderer(GpuScene(ctx, s), s.camera_struct())
    r.params = p
    ragged, _, _ = r.render(want_moments=True)
    assert r.stats.paths == st.paths == 37 * 19 * 3
    # shadow contributions are summed with float atomics: order-dependent
    np.testing.assert_allclose(ragged, a, rtol=1e-5, atol=1e-7)
    assert_path_level(a, b)


def test_depth_one_paths(ctx):
    """max depth 1: the camera vertex only (emission seen directly and its
    next-event estimate)."""
    s = workloads.cornell_box(32, 32)
    a, b, st, o = render_both(ctx, s, render_params(2, 2, 0.5, 1, 5))
    assert_path_level(a, b)
    assert st.extension_rays <= o["rays"]


@pytest.mark.parametrize("semantics", [_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL])
def test_scene_without_lights_is_black(ctx, semantics):
    s = workloads.cornell_box(24, 24)
    s.lights = []
    a, b, st, _ = render_both(ctx, s, render_params(2, 2, 0.5, 8, 2, semantics=semantics))
    assert not a.any() and not b.any()
    assert st.paths == 24 * 24 * 4 and st.nonfinite == 0


@pytest.mark.parametrize("semantics", [_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL])
def test_environment_without_geometry(ctx, semantics):
    """No primitives at all: every camera ray leaves to the environment map,
    which both sides look up in the same direction."""
    s = SceneData()
    rng = np.random.default_rng(8)
    s.env = rng.uniform(0.1, 2.0, (16, 32, 3)).astype(np.float32)
    s.env_mapping = _abi.ENV_LATLONG
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1, 1, 1))]
    s.camera = dict(eye=(0, 0, 0), look_at=(0, 0, -1), up=(0, 1, 0), fov=1.2, width=20, height=12)
    a, b, st, _ = render_both(ctx, s, render_params(2, 2, 0.5, 4, 6, semantics=semantics))
    assert a.min() > 0
    assert_path_level(a, b)
    assert st.paths == 20 * 12 * 4 and st.nonfinite == 0
