"""Neural path guiding: the network kernels against the FP64 restatement
(oracle/guide_ref.py), training, and the guided estimator against the plain
physical one.

CPU tests pin the restatement itself (its gradient against finite
differences, its mixture's normalisation); GPU tests compare the tcgen05
kernels with it and check what guiding does to a render."""
import math

import numpy as np
import pytest

from oracle import guide_ref as gr


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def random_inputs(n, bounds, rng):
    lo, hi = np.asarray(bounds[:3]), np.asarray(bounds[3:])
    p = lo + rng.random((n, 3)) * (hi - lo)
    return np.concatenate([p, _unit(rng.normal(size=(n, 3))), _unit(rng.normal(size=(n, 3)))], 1).astype(np.float32)


def random_samples(n, bounds, rng):
    x = random_inputs(n, bounds, rng)
    wi = _unit(rng.normal(size=(n, 3)))
    w = rng.exponential(1.0, size=(n, 1))
    return np.concatenate([x, wi, w], 1).astype(np.float32)


def init_weights(seed=0):
    rng = np.random.default_rng(seed)
    parts = []
    for (a, b), s in zip(gr.SHAPES, (1, 1, 1, 0.1)):
        lim = math.sqrt(6 / b) * s
        parts.append(rng.uniform(-lim, lim, a * b))
    return np.concatenate(parts).astype(np.float32)


BOUNDS = np.array([-1.0, 0.0, -2.0, 3.0, 2.0, 1.0], np.float32)


# ------------------------------------------------------------------ CPU ----
def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    w = init_weights(1).astype(np.float64)
    s = random_samples(40, BOUNDS, rng)
    _, g = gr.loss_and_grad(w, s, BOUNDS, bf16=False)
    for i in rng.choice(len(w), 24, replace=False):
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        lp, _ = gr.loss_and_grad(wp, s, BOUNDS, bf16=False)
        lm, _ = gr.loss_and_grad(wm, s, BOUNDS, bf16=False)
        assert g[i] == pytest.approx((lp - lm) / (2 * h), rel=1e-4, abs=1e-9)


def test_reference_mixture_integrates_to_one():
    rng = np.random.default_rng(2)
    mix = gr.mixture(init_weights(2) * 4, random_inputs(3, BOUNDS, rng), BOUNDS, bf16=False)
    n = 200000
    k = np.arange(n) + 0.5
    z = 1 - 2 * k / n
    phi = np.pi * (1 + 5 ** 0.5) * k
    r = np.sqrt(1 - z * z)
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    for m in mix:
        integral = gr.mixture_pdf(np.repeat(m[None], n, 0), d).mean() * 4 * np.pi
        assert integral == pytest.approx(1.0, rel=2e-3)


def test_encoding_layout():
    x = np.array([[0.5, 1.0, -0.5, 0, 0, 1, 0, 0, 1]], np.float32)
    e = gr.encode(x, BOUNDS).numpy()[0]
    assert e.shape == (208,)
    # position x normalised to 0.375: band 0 of coordinate 0 is sin/cos(0.375 pi)
    assert e[0] == pytest.approx(math.sin(0.375 * math.pi)) and e[1] == pytest.approx(math.cos(0.375 * math.pi))
    # outgoing direction +z: theta = 0 -> the first theta bin is the largest
    assert np.argmax(e[144:176]) == 0


# ------------------------------------------------------------------ GPU ----
@pytest.fixture
def guide(ctx):
    from renderer_gb300.guiding import Guide
    g = Guide(ctx, BOUNDS, seed=3)
    yield g
    g.close()


@pytest.mark.gpu
def test_guide_eval_matches_reference(guide):
    rng = np.random.default_rng(4)
    w = init_weights(4) * 3  # larger weights: non-trivial mixtures
    guide.set_weights(w)
    assert np.array_equal(guide.weights(), w)
    # enough rows for every warpgroup of every block to run several tiles,
    # and a ragged last tile
    x = random_inputs(152 * 6 * 128 * 3 + 77, BOUNDS, rng)
    got = guide.eval(x)
    ref = gr.mixture(w, x, BOUNDS, bf16=True)
    # Both sides round the same tensors to bfloat16; FP32 and FP64 sums can
    # still round a hidden activation to neighbouring bfloat16 values (one
    # ulp, 2^-8 relative), which these large weights amplify in a few rows.
    dpi = np.abs(got[:, :8] - ref[:, :8])
    assert np.quantile(dpi, 0.99) < 1e-4 and dpi.max() < 3e-2
    gl, rl = got[:, 8:].reshape(-1, 8, 4), ref[:, 8:].reshape(-1, 8, 4)
    cosang = (gl[..., :3] * rl[..., :3]).sum(-1)
    assert np.quantile(cosang, 0.01) > 0.99999 and cosang.min() > 0.99
    dk = np.abs(gl[..., 3] / rl[..., 3] - 1)
    assert np.quantile(dk, 0.99) < 1e-3 and dk.max() < 0.1
    d = _unit(rng.normal(size=(len(x), 3)))
    dq = np.abs(gr.mixture_pdf(got, d) / gr.mixture_pdf(ref, d) - 1)
    assert np.quantile(dq, 0.99) < 1e-3


@pytest.mark.gpu
def test_guide_gradient_matches_reference(guide):
    rng = np.random.default_rng(5)
    w = init_weights(5) * 2
    guide.set_weights(w)
    s = random_samples(4096 + 333, BOUNDS, rng)
    g, loss = guide.gradient(s)
    lr, gref = gr.loss_and_grad(w, s, BOUNDS, bf16=True)
    assert loss == pytest.approx(lr, rel=2e-3)
    o = 0
    for a, b in gr.SHAPES:
        x, y = g[o:o + a * b].astype(np.float64), gref[o:o + a * b]
        o += a * b
        cos = x @ y / (np.linalg.norm(x) * np.linalg.norm(y))
        rel = np.linalg.norm(x - y) / np.linalg.norm(y)
        assert cos > 0.999 and rel < 3e-2, ((a, b), cos, rel)


@pytest.mark.gpu
def test_guide_learns_a_lobe(guide):
    """Samples drawn from one vMF lobe at every position: the trained mixture
    puts its mass there."""
    rng = np.random.default_rng(6)
    mu = _unit(np.array([0.3, 0.5, -0.8]))
    kappa = 40.0

    def vmf(n):
        u1, u2 = rng.random(n), rng.random(n)
        w = 1 + np.log(u1 + (1 - u1) * np.exp(-2 * kappa)) / kappa
        t = _unit(np.cross(mu, [1.0, 0, 0]))
        b = np.cross(mu, t)
        s = np.sqrt(np.clip(1 - w * w, 0, 1))
        return (s * np.cos(2 * np.pi * u2))[:, None] * t + (s * np.sin(2 * np.pi * u2))[:, None] * b + w[:, None] * mu

    losses = []
    for it in range(300):
        x = random_inputs(4096, BOUNDS, rng)
        s = np.concatenate([x, vmf(4096), np.ones((4096, 1))], 1).astype(np.float32)
        losses.append(guide.train_step(s, 1e-2))
    assert losses[-1] < losses[0] - 2.0
    x = random_inputs(256, BOUNDS, rng)
    q = gr.mixture_pdf(guide.eval(x), np.repeat(mu[None], 256, 0))
    true_peak = kappa / (2 * np.pi * (1 - np.exp(-2 * kappa)))
    assert np.median(q) > 0.3 * true_peak


def _small_rooms(ctx, w=64, h=48, quads=24):
    from renderer_gb300.runtime import GpuScene
    from renderer_gb300.workloads import two_rooms
    data = two_rooms(w, h, mesh_quads=quads)
    return GpuScene(ctx, data), data.camera_struct()


@pytest.mark.gpu
def test_guided_render_needs_physical_semantics(ctx):
    from renderer_gb300 import GbrtError
    from renderer_gb300.guiding import guide_params, render_guided
    from renderer_gb300.scene import render_params
    sc, cam = _small_rooms(ctx)
    with pytest.raises(GbrtError):
        render_guided(sc, cam, render_params(1, 1, 0.5, 8, 0), None, guide_params(passes=1))


@pytest.mark.gpu
def test_guide_off_matches_plain_physical_render(ctx):
    """guide = NULL is the physical estimator: one pass equals gbrt_render
    with the pass's seed... statistically; many passes converge to it."""
    from renderer_gb300.guiding import guide_params, render_guided
    from renderer_gb300.runtime import PerPixelRenderer
    from renderer_gb300.workloads import two_rooms_params
    sc, cam = _small_rooms(ctx)
    prm = two_rooms_params(4, 4, seed=1)
    film, st = render_guided(sc, cam, prm, None, guide_params(passes=16))
    assert st.passes == 16 and st.train_steps == 0
    r = PerPixelRenderer(sc, cam, {"pt-x-samples": 16, "pt-y-samples": 16, "pt-termination-prob": 0.5},
                         seed=7, max_depth=12)
    r.params.semantics = 1
    plain = r.render()
    assert film.mean() == pytest.approx(plain.mean(), rel=0.03)


@pytest.mark.gpu
def test_guided_render_is_unbiased_and_helps(ctx):
    """The two rooms, lit through the door: a guide trained online by the
    renderer (512 Adam steps on its own radiance samples) leaves the image's
    expectation unchanged and, at equal samples per pixel, lowers the relMSE
    against a 16,384-spp render."""
    from renderer_gb300.guiding import Guide, guide_params, render_guided, scene_bounds
    from renderer_gb300.workloads import two_rooms_params
    sc, cam = _small_rooms(ctx, 128, 96, 24)
    ref, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=11), None, guide_params(passes=256))
    plain, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=12), None, guide_params(passes=4))
    def relmse(x):
        return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))

    ratios = []
    for seed in (1, 2, 3, 4):
        g = Guide(ctx, scene_bounds(sc), seed=seed)
        gp = guide_params(0.5, passes=16, train_passes=16, steps_per_pass=32, batch_samples=1 << 16,
                          learning_rate=1e-2)
        trained, st = render_guided(sc, cam, two_rooms_params(8, 8, seed=13 + 2 * seed), g, gp)
        guided, st2 = render_guided(sc, cam, two_rooms_params(8, 8, seed=14 + 2 * seed), g, guide_params(0.5, passes=4))
        g.close()
        assert st.train_steps == 512 and st.train_samples > 0 and st2.train_steps == 0
        assert trained.mean() == pytest.approx(ref.mean(), rel=0.02)
        assert guided.mean() == pytest.approx(ref.mean(), rel=0.02)
        ratios.append(relmse(guided) / relmse(plain))
    # Training is not bit-reproducible (samples and gradients are gathered
    # with atomics, and Adam turns the last-bit differences of near-zero
    # gradients into different steps) and its result varies: over guide seeds
    # 1-8 in one run the ratio was 0.52-1.07 (median 0.67), and a guide's
    # ratio once reached 1.41 (this radiance target sends guided directions
    # past the glossy floor's lobe; the product target, tested below, does
    # not). Of four guides trained independently, the best one helps and
    # none hurts badly.
    assert min(ratios) < 0.85 and max(ratios) < 1.6, ratios


@pytest.mark.gpu
def test_product_target_is_unbiased_and_helps(ctx):
    """GBRT_GUIDE_PRODUCT (the guide learns BSDF x radiance x cos): the same
    two rooms, the same expectation, and at equal samples per pixel a lower
    relMSE than plain sampling."""
    from renderer_gb300 import _abi
    from renderer_gb300.guiding import Guide, guide_params, render_guided, scene_bounds
    from renderer_gb300.workloads import two_rooms_params
    sc, cam = _small_rooms(ctx, 128, 96, 24)
    ref, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=21), None, guide_params(passes=256))
    plain, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=22), None, guide_params(passes=4))

    def relmse(x):
        return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))

    ratios = []
    for seed in (1, 2):
        g = Guide(ctx, scene_bounds(sc), seed=seed)
        gp = guide_params(0.5, passes=16, train_passes=16, steps_per_pass=32, batch_samples=1 << 16,
                          learning_rate=1e-2, flags=_abi.GUIDE_PRODUCT)
        trained, st = render_guided(sc, cam, two_rooms_params(8, 8, seed=23 + 2 * seed), g, gp)
        guided, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=24 + 2 * seed), g, guide_params(0.5, passes=4))
        g.close()
        assert st.train_steps == 512 and st.train_samples > 0
        assert trained.mean() == pytest.approx(ref.mean(), rel=0.02)
        assert guided.mean() == pytest.approx(ref.mean(), rel=0.02)
        ratios.append(relmse(guided) / relmse(plain))
    assert min(ratios) < 0.85 and max(ratios) < 1.2, ratios


@pytest.mark.gpu
def test_late_passes_keep_the_expectation(ctx):
    """late_pass_samples: training passes of 2 x 2 samples per pixel, then
    passes of 64 samples (64 x 1 strata). With equal pass weights the film is
    the plain mean of all samples, unbiased by construction; the path count
    adds up and the image keeps the plain estimator's expectation. The
    default inverse-deviation weights combine passes of different sizes by
    their means (looser bound: their weights depend on the passes). A render
    that does not train takes the late size for every pass."""
    from renderer_gb300 import _abi
    from renderer_gb300.guiding import Guide, guide_params, render_guided, scene_bounds
    from renderer_gb300.workloads import two_rooms_params
    sc, cam = _small_rooms(ctx, 96, 64, 24)
    npix = 96 * 64
    ref, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=31), None, guide_params(passes=256))
    for flags, tol, seed in ((_abi.GUIDE_EQUAL_WEIGHTS, 0.02, 32), (0, 0.04, 34)):
        g = Guide(ctx, scene_bounds(sc), seed=3)
        gp = guide_params(0.5, passes=14, train_passes=8, steps_per_pass=8, batch_samples=1 << 16,
                          learning_rate=1e-2, late_pass_samples=64, flags=flags)
        img, st = render_guided(sc, cam, two_rooms_params(2, 2, seed=seed), g, gp)
        assert st.passes == 14 and st.train_steps == 64
        assert st.paths == npix * (8 * 4 + 6 * 64)
        assert img.mean() == pytest.approx(ref.mean(), rel=tol)
        if flags:
            img2, st2 = render_guided(sc, cam, two_rooms_params(1, 1, seed=33), g,
                                      guide_params(0.5, passes=4, late_pass_samples=64))
            assert st2.paths == npix * 4 * 64 and st2.train_steps == 0
            assert img2.mean() == pytest.approx(ref.mean(), rel=0.03)
        g.close()


@pytest.mark.gpu
def test_async_training_keeps_the_expectation_and_trains(ctx):
    """GBRT_GUIDE_ASYNC_TRAINING: the Adam steps run on a second stream while
    the next pass renders (each pass sampling the weights of the steps two
    passes back). The render keeps its expectation, every step is taken, the
    guide ends with the last step's weights (the same as its FP32 master
    parameters rounded) and helps at equal samples like synchronous
    training."""
    from renderer_gb300 import _abi
    from renderer_gb300.guiding import Guide, guide_params, render_guided, scene_bounds
    from renderer_gb300.workloads import two_rooms_params
    sc, cam = _small_rooms(ctx, 128, 96, 24)
    ref, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=31), None, guide_params(passes=256))
    plain, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=32), None, guide_params(passes=4))

    def relmse(x):
        return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))

    ratios = []
    for seed in (1, 2):
        g = Guide(ctx, scene_bounds(sc), seed=seed)
        w0 = g.weights()
        gp = guide_params(0.5, passes=16, train_passes=16, steps_per_pass=32, batch_samples=1 << 16,
                          learning_rate=1e-2, flags=_abi.GUIDE_PRODUCT | _abi.GUIDE_ASYNC_TRAINING)
        trained, st = render_guided(sc, cam, two_rooms_params(8, 8, seed=33 + 2 * seed), g, gp)
        assert st.train_steps == 512 and st.train_samples > 0 and st.passes == 16
        state = g.get_state()
        assert state["step"] == 512 and not np.array_equal(state["params"], w0)
        # the inference copy is the last step's weights: evaluating the guide
        # equals evaluating its master parameters set as weights
        x = np.concatenate([np.random.default_rng(seed).uniform(0, 1, (256, 3)) * 2,
                            np.tile([0, 1, 0], (256, 1)), np.tile([0, 0, 1], (256, 1))], 1).astype(np.float32)
        e1 = g.eval(x)
        h = Guide(ctx, scene_bounds(sc), seed=9)
        h.set_weights(state["params"])
        np.testing.assert_allclose(e1, h.eval(x), rtol=1e-5, atol=1e-6)
        h.close()
        guided, _ = render_guided(sc, cam, two_rooms_params(8, 8, seed=34 + 2 * seed), g, guide_params(0.5, passes=4))
        g.close()
        assert trained.mean() == pytest.approx(ref.mean(), rel=0.02)
        assert guided.mean() == pytest.approx(ref.mean(), rel=0.02)
        ratios.append(relmse(guided) / relmse(plain))
    assert min(ratios) < 0.85 and max(ratios) < 1.2, ratios
