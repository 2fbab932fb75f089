"""gbrt_render_device_noalloc: the render entry point for callers that cannot
call cudaMalloc during a render (their device memory belongs to their own pool
or a fixed budget, or their frame loop cannot take cudaMalloc's
synchronisation). Its wavefront state lives in one fixed device array instead
of per-call allocations.

The test renders the same frame through the existing gbrt_render_device and
then twice in a row through the no-allocation entry point (whose array keeps
the previous call's contents), and requires the same film each time. Both
paths run the same kernels on the same per-sample random numbers; only the
batch size and the float order of the shadow-ray additions differ, so the
films agree to rtol 1e-5 (the tolerance of the closed-form GPU tests).

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_render_matches_allocating_render(ctx):
    import torch

    import renderer_gb300 as rg
    from renderer_gb300 import GpuScene, _abi, workloads

    s = workloads.cornell_box(96, 64)
    gs = GpuScene(ctx, s)
    cam = s.camera_struct()
    params = workloads.cornell_params(max_depth=8, seed=21)
    H, W = cam.height, cam.width
    lib = rg.lib()

    def buffers():
        return (torch.zeros(H * W * 3, dtype=torch.float32, device="cuda"),
                torch.zeros(H * W * 3, dtype=torch.float64, device="cuda"),
                torch.zeros(H * W * 3, dtype=torch.float64, device="cuda"))

    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    film, fsum, fsq = buffers()
    st = _abi.Stats()
    rg.check(lib.gbrt_render_device(gs.handle, C.byref(cam), C.byref(params), ptr(film), ptr(fsum), ptr(fsq),
                                    C.byref(st)), ctx.handle)
    torch.cuda.synchronize()
    ref = film.cpu().numpy()
    ref_sq = fsq.cpu().numpy()
    assert st.paths == H * W * 16 and np.isfinite(ref).all() and ref.max() > 0

    for call in range(2):
        f2, s2, q2 = buffers()
        f2.fill_(-1.0)  # stale output must be overwritten
        st2 = _abi.Stats()
        rg.check(lib.gbrt_render_device_noalloc(gs.handle, C.byref(cam), C.byref(params), ptr(f2), ptr(s2), ptr(q2),
                                                C.byref(st2)), ctx.handle)
        torch.cuda.synchronize()
        out = f2.cpu().numpy()
        np.testing.assert_allclose(out, ref, rtol=1e-5, atol=1e-6, err_msg="call %d" % call)
        np.testing.assert_allclose(q2.cpu().numpy(), ref_sq, rtol=1e-5, atol=1e-6)
        assert st2.paths == st.paths and st2.extension_rays == st.extension_rays
        assert st2.shadow_rays == st.shadow_rays and st2.nonfinite == 0


def test_noalloc_rejects_oversized_batches(ctx):
    import torch

    import renderer_gb300 as rg
    from renderer_gb300 import GpuScene, _abi, workloads

    s = workloads.cornell_box(16, 16)
    gs = GpuScene(ctx, s)
    cam = s.camera_struct()
    params = workloads.cornell_params(max_depth=5)
    params.batch_paths = _abi.NOALLOC_MAX_BATCH + 1
    f = torch.zeros(16 * 16 * 3, dtype=torch.float32, device="cuda")
    d = torch.zeros(16 * 16 * 3, dtype=torch.float64, device="cuda")
    lib = rg.lib()
    st = lib.gbrt_render_device_noalloc(gs.handle, C.byref(cam), C.byref(params), C.c_void_p(f.data_ptr()),
                                        C.c_void_p(d.data_ptr()), None, None)
    assert st == _abi.ERR_INVALID_ARG
    assert b"65536" in lib.gbrt_last_error(ctx.handle)
    # the sum buffer is required: it scales with the image
    params.batch_paths = 0
    st = lib.gbrt_render_device_noalloc(gs.handle, C.byref(cam), C.byref(params), C.c_void_p(f.data_ptr()), None,
                                        None, None)
    assert st == _abi.ERR_INVALID_ARG
