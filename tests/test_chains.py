"""The Markov-chain renderers: MetropolisRenderer and
EnergyRedistributionRenderer (gbrt_render_mlt, gbrt_render_erpt).

CPU: the oracle's restatement keeps the identities of the renderer's
estimators — every Metropolis iteration deposits luminance b / mutations in
total, so the film's luminance sums to iterations x b / mutations; with one
chain the start is the renderer's own bootstrap choice; runs are
deterministic per seed. GPU: the CUDA chains equal the oracle's chain by chain
(same keys of the counter-based stream), the film's identities hold at full
size, and the Metropolis image has the per-pixel renderer's image shape."""
import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import GbrtError, GpuScene, _abi, workloads
from renderer_gb300.chains import EnergyRedistributionRenderer, MetropolisRenderer, erpt_params, mlt_params
from renderer_gb300.scene import render_params


def lum(film):
    f = film.astype(np.float64)
    return .299 * f[..., 2] + .587 * f[..., 1] + .114 * f[..., 0]


def test_oracle_mlt_deposits_b_per_iteration():
    s = workloads.cornell_box(24, 24)
    r = OracleScene(s).render_mlt(s.camera_struct(), render_params(1, 1, 0.0, 5, 3), mlt_params(16, 2000), chains=48)
    assert r["chains"] == 48 and r["mutations"] == 48 * (16 * 24 * 24 // 48)
    assert r["paths"] == 2000 + r["mutations"]
    assert 0 < r["accepted"] < r["mutations"]
    assert lum(r["film"]).sum() == pytest.approx(r["mutations"] * r["b"] / 16, rel=1e-5)


def test_oracle_chains_are_deterministic_per_seed():
    s = workloads.cornell_box(16, 16)
    o = OracleScene(s)
    cam = s.camera_struct()
    a = o.render_mlt(cam, render_params(1, 1, 0.0, 5, 1), mlt_params(8, 500), chains=8)["film"]
    b = o.render_mlt(cam, render_params(1, 1, 0.0, 5, 1), mlt_params(8, 500), chains=8)["film"]
    c = o.render_mlt(cam, render_params(1, 1, 0.0, 5, 2), mlt_params(8, 500), chains=8)["film"]
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    e1 = o.render_erpt(cam, render_params(1, 1, 0.0, 5, 1), erpt_params(5, 1, 1))
    e2 = o.render_erpt(cam, render_params(1, 1, 0.0, 5, 1), erpt_params(5, 1, 1))
    assert np.array_equal(e1["film"], e2["film"]) and e1["chains"] == e2["chains"]


def test_oracle_erpt_chain_counts():
    """(int)(u + |c| / (M ed)) chains per initial sample: with ed the mean
    corner-path energy per mutation, about one chain per initial sample; every
    chain makes M mutations."""
    s = workloads.cornell_box(24, 24)
    r = OracleScene(s).render_erpt(s.camera_struct(), render_params(1, 1, 0.0, 5, 4), erpt_params(10, 2, 2))
    n_init = 24 * 24 * 4
    assert r["mutations"] == r["chains"] * 10
    assert r["paths"] == 24 * 24 + n_init + r["mutations"]
    assert 0.3 * n_init < r["chains"] < 3 * n_init
    assert r["ed"] > 0 and np.isfinite(r["film"]).all() and (r["film"] >= 0).all()


def _close_fraction(a, b, rel=2e-3):
    a, b = a.astype(np.float64), b.astype(np.float64)
    return (np.abs(a - b) <= rel * np.maximum(np.abs(b), 1e-3)).all(-1).mean()


@pytest.mark.gpu
def test_mlt_matches_oracle_chain_by_chain(ctx):
    s = workloads.cornell_box(32, 32)
    prm = render_params(1, 1, 0.0, 5, 7)
    mp = mlt_params(16, 3000, 0.1, 0.5, chains=128)
    r = MetropolisRenderer(GpuScene(ctx, s), options={"met-mutations": 16, "met-bootstrap": 3000}, seed=7,
                           max_depth=5, chains=128)
    film = r.render()
    st = r.stats
    o = OracleScene(s).render_mlt(s.camera_struct(), prm, mp, chains=128)
    assert st.normaliser == pytest.approx(o["b"], rel=1e-5)
    assert st.chains == 128 and st.mutations == o["mutations"] and st.paths == o["paths"]
    assert st.accepted == pytest.approx(o["accepted"], rel=0.01)
    assert _close_fraction(film, o["film"]) >= 0.95
    assert film.sum() == pytest.approx(o["film"].sum(), rel=1e-3)
    assert st.nonfinite == 0 and st.kernel_launches > 0 and st.render_ms > 0


def off_axis_cornell(n):
    """The Cornell box seen from slightly off its axis of symmetry, so that
    the rays through pixel corners (ERPT's energy pass) meet no edge exactly."""
    s = workloads.cornell_box(n, n)
    s.camera["eye"] = (0.0137, 1.0123, 3.4)
    s.camera["look_at"] = (0.0041, 0.9931, 0.0)
    return s


@pytest.mark.gpu
def test_erpt_matches_oracle_chain_by_chain(ctx):
    s = off_axis_cornell(32)
    prm = render_params(1, 1, 0.0, 5, 5)
    r = EnergyRedistributionRenderer(GpuScene(ctx, s), options={"erpt-mutations": 12}, seed=5, max_depth=5)
    film = r.render()
    st = r.stats
    o = OracleScene(s).render_erpt(s.camera_struct(), prm, erpt_params(12, 2, 2))
    assert st.normaliser == pytest.approx(o["ed"], rel=1e-6)
    assert st.chains == o["chains"] and st.mutations == o["mutations"] and st.paths == o["paths"]
    assert st.accepted == pytest.approx(o["accepted"], rel=0.01)
    assert _close_fraction(film, o["film"]) >= 0.95
    assert film.sum() == pytest.approx(o["film"].sum(), rel=2e-3)


@pytest.mark.gpu
def test_erpt_batches_of_chains_agree(ctx):
    """Chains split over several wavefronts give the film of one wavefront."""
    s = off_axis_cornell(24)
    gs = GpuScene(ctx, s)
    a = EnergyRedistributionRenderer(gs, options={"erpt-mutations": 6}, seed=2).render()
    r = EnergyRedistributionRenderer(gs, options={"erpt-mutations": 6}, seed=2, batch_chains=700)
    b = r.render()
    assert r.stats.chains > 700
    assert np.allclose(a, b, rtol=1e-5, atol=1e-7)


@pytest.mark.gpu
def test_mlt_full_size_identities_and_image(ctx):
    """The Cornell box at 256 x 256 with the default chain count: luminance
    sums to iterations x b / mutations, and the image, normalised by its mean,
    is the per-pixel renderer's image (8 x 8-pixel blocks)."""
    from renderer_gb300 import PerPixelRenderer
    s = workloads.cornell_box(256, 256)
    gs = GpuScene(ctx, s)
    r = MetropolisRenderer(gs, options={"met-mutations": 64}, seed=11, max_depth=5)
    film = r.render()
    st = r.stats
    assert st.mutations == st.chains * (64 * 256 * 256 // st.chains)
    assert lum(film).sum() == pytest.approx(st.mutations * st.normaliser / 64, rel=1e-4)
    pt = PerPixelRenderer(gs, options={"pt-x-samples": 8, "pt-y-samples": 8}, seed=3, max_depth=5).render()

    def blocks(x):
        y = lum(x).reshape(32, 8, 32, 8).mean((1, 3))
        return y / y.mean()
    bm, bp = blocks(film), blocks(pt)
    bright = bp > 0.2
    assert np.median(np.abs(bm[bright] - bp[bright]) / bp[bright]) < 0.1


def _dark_room(n):
    """The Cornell room without its light: every path carries nothing."""
    s = workloads.cornell_box(n, n)
    s.lights = []
    return s


def test_oracle_chains_on_a_black_scene():
    s = _dark_room(8)
    o = OracleScene(s)
    r = o.render_mlt(s.camera_struct(), render_params(1, 1, 0.0, 5, 1), mlt_params(4, 100), chains=4)
    assert r["b"] == 0 and not r["film"].any()
    e = o.render_erpt(s.camera_struct(), render_params(1, 1, 0.0, 5, 1), erpt_params(3, 1, 1))
    assert e["chains"] == 0 and not e["film"].any()


@pytest.mark.gpu
def test_chain_renderers_on_a_black_scene(ctx):
    s = _dark_room(16)
    gs = GpuScene(ctx, s)
    r = MetropolisRenderer(gs, options={"met-mutations": 4, "met-bootstrap": 200}, chains=64)
    assert not r.render().any() and r.stats.normaliser == 0 and r.stats.nonfinite == 0
    e = EnergyRedistributionRenderer(gs, options={"erpt-mutations": 3})
    assert not e.render().any() and e.stats.chains == 0


@pytest.mark.gpu
def test_chain_renderers_refuse_other_estimators(ctx):
    from renderer_gb300 import check, lib
    import ctypes as C
    s = workloads.cornell_box(8, 8)
    gs = GpuScene(ctx, s)
    cam = s.camera_struct()
    film = np.zeros((8, 8, 3), np.float32)
    st = _abi.ChainStats()
    phys = render_params(1, 1, 0.0, 5, 0, semantics=_abi.SEM_PHYSICAL)
    assert lib().gbrt_render_mlt(gs.handle, C.byref(cam), C.byref(phys), C.byref(mlt_params()),
                                 film.ctypes.data_as(C.c_void_p), C.byref(st)) == _abi.ERR_INVALID_ARG
    assert lib().gbrt_render_erpt(gs.handle, C.byref(cam), C.byref(phys), C.byref(erpt_params()),
                                  film.ctypes.data_as(C.c_void_p), C.byref(st)) == _abi.ERR_INVALID_ARG
    with pytest.raises(GbrtError):
        MetropolisRenderer(gs, options={"met-large-step-prob": 1.5}).render()
    with pytest.raises(GbrtError):
        check(lib().gbrt_render_erpt(gs.handle, C.byref(cam), C.byref(render_params(1, 1, 0.0, 5, 0)),
                                     C.byref(erpt_params(0)), film.ctypes.data_as(C.c_void_p), C.byref(st)),
              ctx.handle)
