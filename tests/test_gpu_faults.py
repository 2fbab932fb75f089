"""Failure paths, driven by the library's host-side fault injection
(gbrt_debug_fault). Nothing here faults, traps or hangs the GPU: an
allocation fails on the host, NaN radiance is planted before accumulation,
the traversal kernels run with a 4-entry stack (their own bounds check
catches the overflow), and the guide's kernels issue no tensor-core products
and give up their bounded wait after 1 ms.

The renderer being replaced meets these conditions with assert
(src/perpixelrenderer.cpp:90-91) or not at all; here each becomes a status
code, and the context keeps working afterwards.
"""
import numpy as np
import pytest

from renderer_gb300 import Context, GbrtError, GpuScene, PerPixelRenderer, _abi, lib, workloads

pytestmark = pytest.mark.gpu


def fault(ctx, kind, arg=0):
    assert lib().gbrt_debug_fault(ctx.handle, kind, arg) == _abi.OK


def render(gs, params, moments=False):
    r = PerPixelRenderer(gs, gs.data.camera_struct())
    r.params = params
    out = r.render(want_moments=moments)
    return out, r.stats


@pytest.fixture
def fctx(gbrt_built):
    """A context of its own, so that a fault never leaks into other tests."""
    c = Context(0)
    yield c
    fault(c, _abi.FAULT_NONE)
    c.close()


def test_allocation_failure_returns_oom_and_the_context_recovers(fctx):
    s = workloads.cornell_box(32, 32)
    gs = GpuScene(fctx, s)
    params = workloads.cornell_params(max_depth=5, seed=1)
    clean, _ = render(gs, params)
    # the render's first buffer
    fault(fctx, _abi.FAULT_ALLOC, 0)
    with pytest.raises(GbrtError) as ei:
        render(gs, params)
    assert ei.value.status == _abi.ERR_OOM
    # one in the middle of its buffers
    fault(fctx, _abi.FAULT_ALLOC, 7)
    with pytest.raises(GbrtError) as ei:
        render(gs, params)
    assert ei.value.status == _abi.ERR_OOM
    # the fault is one-shot: the next render works and gives the same image
    again, st = render(gs, params)
    np.testing.assert_allclose(again, clean, rtol=1e-6, atol=1e-7)
    assert st.paths == 32 * 32 * 16
    # scene creation: a failure part-way frees what it made; the next works
    fault(fctx, _abi.FAULT_ALLOC, 3)
    with pytest.raises(GbrtError) as ei:
        GpuScene(fctx, s)
    assert ei.value.status == _abi.ERR_OOM
    gs2 = GpuScene(fctx, s)
    np.testing.assert_allclose(render(gs2, params)[0], clean, rtol=1e-6, atol=1e-7)


def test_nan_radiance_is_counted_and_dropped(fctx):
    s = workloads.cornell_box(40, 40)
    gs = GpuScene(fctx, s)
    params = workloads.cornell_params(max_depth=6, seed=5)
    params.x_samples = params.y_samples = 1
    clean, st0 = render(gs, params)
    assert st0.nonfinite == 0
    every = 5
    fault(fctx, _abi.FAULT_NAN, every)
    (film, fsum, fsq), st = render(gs, params, moments=True)
    n = 40 * 40
    # one sample per pixel: path index == pixel index
    hit = np.arange(n) % every == 0
    assert st.nonfinite == hit.sum()
    assert np.isfinite(film).all() and np.isfinite(fsum).all() and np.isfinite(fsq).all()
    f, c = film.reshape(n, 3), clean.reshape(n, 3)
    assert (f[hit] == 0).all()
    np.testing.assert_allclose(f[~hit], c[~hit], rtol=1e-6, atol=1e-7)
    # the physical estimator drops them the same way
    params.semantics = _abi.SEM_PHYSICAL
    _, stp = render(gs, params)
    assert stp.nonfinite == hit.sum()
    fault(fctx, _abi.FAULT_NAN, 0)
    assert render(gs, params)[1].nonfinite == 0


def test_traversal_stack_overflow_returns_numeric(fctx):
    s = workloads.icosphere_scene(levels=4, width=32, height=32, env_size=(64, 32))
    gs = GpuScene(fctx, s)
    params = workloads.cornell_params(max_depth=4, seed=2)
    clean, _ = render(gs, params)
    fault(fctx, _abi.FAULT_SMALL_STACK, 1)
    with pytest.raises(GbrtError) as ei:
        render(gs, params)
    assert ei.value.status == _abi.ERR_NUMERIC
    assert "stack" in str(ei.value)
    fault(fctx, _abi.FAULT_SMALL_STACK, 0)
    again, st = render(gs, params)
    np.testing.assert_allclose(again, clean, rtol=1e-6, atol=1e-7)
    assert st.nonfinite == 0


def test_guide_wait_timeout_returns_timeout_and_frees_tensor_memory(fctx):
    from renderer_gb300.guiding import Guide, guide_params, render_guided

    rng = np.random.default_rng(3)
    box = np.array([-1, 0, -1, 1, 2, 1], np.float32)

    def unit(v):
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    n = 4096
    x = np.concatenate([rng.uniform(box[:3], box[3:], (n, 3)), unit(rng.normal(size=(n, 3))),
                        unit(rng.normal(size=(n, 3)))], 1).astype(np.float32)
    samples = np.concatenate([x, unit(rng.normal(size=(n, 3))), rng.exponential(1.0, (n, 1))], 1).astype(np.float32)
    guide = Guide(fctx, box, seed=4)
    want = guide.eval(x)
    g0, l0 = guide.gradient(samples)
    w0 = guide.weights()
    fault(fctx, _abi.FAULT_GUIDE_WAIT, 1_000_000)  # 1 ms
    for call in (lambda: guide.eval(x), lambda: guide.gradient(samples), lambda: guide.train_step(samples)):
        with pytest.raises(GbrtError) as ei:
            call()
        assert ei.value.status == _abi.ERR_TIMEOUT
    # no gradient reached the weights
    np.testing.assert_array_equal(guide.weights(), w0)
    # a guided render that trains and samples the guide reports the timeout
    s = workloads.cornell_box(24, 24)
    gs = GpuScene(fctx, s)
    prm = workloads.cornell_params(max_depth=5, seed=6)
    prm.semantics = _abi.SEM_PHYSICAL
    prm.x_samples = prm.y_samples = 1
    gp = guide_params(passes=3, train_passes=2, steps_per_pass=1, batch_samples=4096)
    with pytest.raises(GbrtError) as ei:
        render_guided(gs, s.camera_struct(), prm, guide, gp)
    assert ei.value.status == _abi.ERR_TIMEOUT
    # Cleared: the kernels allocate tensor memory again (which would wait
    # forever had the timed-out launches kept theirs) and compute what they
    # computed before the fault.
    fault(fctx, _abi.FAULT_GUIDE_WAIT, 0)
    guide.set_weights(w0)
    np.testing.assert_array_equal(guide.eval(x), want)
    g1, l1 = guide.gradient(samples)
    np.testing.assert_allclose(g1, g0, rtol=1e-4, atol=1e-6 * np.abs(g0).max())
    assert l1 == pytest.approx(l0, rel=1e-5)
    film, st = render_guided(gs, s.camera_struct(), prm, guide, gp)
    assert np.isfinite(film).all() and st.passes == 3


def test_fault_arguments_are_checked(fctx):
    L = lib()
    assert L.gbrt_debug_fault(fctx.handle, 99, 0) == _abi.ERR_INVALID_ARG
    assert L.gbrt_debug_fault(fctx.handle, _abi.FAULT_ALLOC, -1) == _abi.ERR_INVALID_ARG
    assert L.gbrt_debug_fault(fctx.handle, _abi.FAULT_GUIDE_WAIT, 2_000_000_000) == _abi.ERR_INVALID_ARG
    assert L.gbrt_debug_fault(None, _abi.FAULT_NONE, 0) == _abi.ERR_INVALID_ARG
