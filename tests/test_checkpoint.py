"""Checkpoint and resume (no counterpart in the renderer, which accumulates
one image per process): a render in passes continued from saved FP64 sums
(gbrt_render_passes), and guide training continued from a saved optimizer
state (gbrt_guide_get_state / gbrt_guide_set_state).

Resumed and uninterrupted runs trace the same paths with the same random
numbers and add them in the same per-pixel order; they may differ only in
the order in which a vertex's shadow rays add into its path's radiance
(float atomics), hence the 1e-6 relative tolerance on FP64 sums. Training
resumed from a checkpoint takes the same Adam steps on the same samples; its
gradients are summed with float atomics, hence rtol 1e-4 on the weights."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _passes(ctx, gs, cam, params, first, n, film, fsum, fsq):
    import renderer_gb300 as rg
    from renderer_gb300 import _abi
    st = _abi.Stats()
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    rg.check(rg.lib().gbrt_render_passes(gs.handle, C.byref(cam), C.byref(params), first, n, ptr(film), ptr(fsum),
                                         ptr(fsq), C.byref(st)), ctx.handle)
    return st


def test_render_resumed_from_saved_sums_equals_one_call(ctx):
    import torch

    from renderer_gb300 import GpuScene, workloads
    s = workloads.cornell_box(64, 48)
    gs = GpuScene(ctx, s)
    cam = s.camera_struct()
    params = workloads.cornell_params(max_depth=8, seed=5)
    params.x_samples = params.y_samples = 2
    n3 = 64 * 48 * 3

    def bufs():
        return (torch.full((n3,), -1.0, dtype=torch.float32, device="cuda"),
                torch.full((n3,), 7.0, dtype=torch.float64, device="cuda"),   # stale contents: pass 0 clears them
                torch.full((n3,), 7.0, dtype=torch.float64, device="cuda"))

    f, sm, sq = bufs()
    st = _passes(ctx, gs, cam, params, 0, 6, f, sm, sq)
    one = (f.cpu().numpy(), sm.cpu().numpy(), sq.cpu().numpy())
    assert st.paths == 6 * 64 * 48 * 4 and st.nonfinite == 0
    # first two passes, checkpoint to host memory, resume into fresh buffers
    f, sm, sq = bufs()
    st_a = _passes(ctx, gs, cam, params, 0, 2, f, sm, sq)
    ck = (sm.cpu().numpy().copy(), sq.cpu().numpy().copy())
    del f, sm, sq
    f, sm, sq = bufs()
    sm.copy_(torch.from_numpy(ck[0]))
    sq.copy_(torch.from_numpy(ck[1]))
    st_b = _passes(ctx, gs, cam, params, 2, 4, f, sm, sq)
    two = (f.cpu().numpy(), sm.cpu().numpy(), sq.cpu().numpy())
    assert st_a.paths + st_b.paths == st.paths
    np.testing.assert_allclose(two[1], one[1], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(two[2], one[2], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(two[0], one[0], rtol=1e-6, atol=1e-9)
    # the film is the mean over all passes so far
    np.testing.assert_allclose(one[0], one[1] / (6 * 4), rtol=1e-6, atol=1e-9)
    # the passes draw independent samples: another seed gives another image
    # of the same mean (24 spp over 3,072 pixels: a few percent apart at most)
    params.seed = 77
    f, sm, sq = bufs()
    _passes(ctx, gs, cam, params, 0, 6, f, sm, sq)
    other = f.cpu().numpy()
    assert not np.array_equal(other, one[0])
    assert other.mean() == pytest.approx(float(one[0].mean()), rel=0.06)


def test_render_passes_refuses_bad_arguments(ctx):
    import torch

    import renderer_gb300 as rg
    from renderer_gb300 import GpuScene, _abi, workloads
    s = workloads.cornell_box(16, 16)
    gs = GpuScene(ctx, s)
    cam = s.camera_struct()
    p = workloads.cornell_params(max_depth=4, seed=1)
    t = torch.zeros(16 * 16 * 3, dtype=torch.float64, device="cuda")
    f = torch.zeros(16 * 16 * 3, dtype=torch.float32, device="cuda")
    L = rg.lib()
    for first, n, sums in ((-1, 1, t), (0, 0, t), (0, 1, None)):
        st = L.gbrt_render_passes(gs.handle, C.byref(cam), C.byref(p), first, n, C.c_void_p(f.data_ptr()),
                                  None if sums is None else C.c_void_p(sums.data_ptr()), None, None)
        assert st == _abi.ERR_INVALID_ARG


def test_guide_training_resumes_from_its_state(ctx):
    from renderer_gb300.guiding import Guide
    from tests.test_guide import BOUNDS, random_samples
    rng = np.random.default_rng(4)
    batches = [random_samples(8192, BOUNDS, rng) for _ in range(7)]
    a = Guide(ctx, BOUNDS, seed=1)
    for b in batches[:4]:
        a.train_step(b)
    ck = a.get_state()
    assert ck["step"] == 4 and np.abs(ck["adam_v"]).max() > 0
    for b in batches[4:]:
        a.train_step(b)
    wa = a.weights()
    b_ = Guide(ctx, BOUNDS, seed=2)  # another initialisation, replaced by the checkpoint
    b_.set_state(ck)
    st = b_.get_state()
    assert st["step"] == 4
    np.testing.assert_array_equal(st["params"], ck["params"])
    np.testing.assert_array_equal(st["adam_m"], ck["adam_m"])
    for b in batches[4:]:
        b_.train_step(b)
    np.testing.assert_allclose(b_.weights(), wa, rtol=1e-4, atol=1e-6)
    # a state with a NaN is refused and leaves the guide as it was
    bad = dict(ck, params=ck["params"].copy())
    bad["params"][3] = np.nan
    from renderer_gb300 import GbrtError
    with pytest.raises(GbrtError):
        b_.set_state(bad)
    assert b_.get_state()["step"] == 7
