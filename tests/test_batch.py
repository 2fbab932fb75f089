"""Batches of renders (gbrt_render_batch, gbrt_batch_autotune) and the seeded
64-scene batch workload.

CPU: the workload generator is deterministic and draws what it promises
(triangle counts, materials, lights, resolutions, samples per pixel). GPU:
every film of a batch equals the film of the same job rendered alone by
gbrt_render (same wavefront size; up to the order of float additions of
shadow rays), whatever the number of streams; batch
jobs match the oracle path by path; the statistics add up; autotuning keeps
its choice on the context; bad jobs are refused with a status."""
import ctypes as C

import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import GbrtError, GpuScene, PerPixelRenderer, _abi, workloads
from renderer_gb300.scene import render_params

SMALL = (6, 8, 9)       # scenes of the batch with about 15,000 triangles
MIXED = (3, 6, 8, 9, 11)


def shrunk(i, res, xs, ys, seed=None):
    s, p = workloads.batch_scene(i)
    s.camera["width"] = s.camera["height"] = res
    return s, render_params(xs, ys, p.termination_prob, p.max_depth, p.seed if seed is None else seed)


def test_batch_workload_is_seeded_and_in_range():
    a, pa = workloads.batch_scene(8)
    b, pb = workloads.batch_scene(8)
    assert np.array_equal(a.tri_pos, b.tri_pos) and a.spheres == b.spheres and a.lights == b.lights
    assert (pa.x_samples, pa.y_samples) == (pb.x_samples, pb.y_samples)
    c, _ = workloads.batch_scene(8, seed=1)
    assert not np.array_equal(a.tri_pos, c.tri_pos)
    for i in SMALL + (3, 11):
        s, p = workloads.batch_scene(i)
        assert 10_000 * 0.9 <= s.n_tri() <= 2_000_000 * 1.05
        assert 1 <= len(s.lights) <= 4 and all(5 <= l["intensity"][0] <= 50 for l in s.lights)
        assert 2 <= len(s.spheres) <= 8
        assert s.camera["width"] == s.camera["height"] in workloads.BATCH_RESOLUTIONS
        assert 4 <= p.x_samples * p.y_samples <= 256
        assert s.flags & _abi.SCENE_GPU_BUILD
        kinds = {m["type"] for m in s.materials[1:]}
        assert kinds <= {_abi.MAT_DIFFUSE, _abi.MAT_MIRROR, _abi.MAT_TRANSPARENT, _abi.MAT_BLINN}
        for m in s.materials:
            if m["type"] == _abi.MAT_BLINN:
                assert 10 <= m["exponent"] <= 500
        # every mesh vertex inside the box
        P = s.tri_pos.reshape(-1, 3)
        assert P.min(0)[1] > -0.5 and P.max(0)[1] < 3.5


@pytest.mark.gpu
def test_batch_equals_individual_renders(ctx):
    from renderer_gb300.batch import BatchJob, render_batch
    scenes = [shrunk(i, 48 + 16 * k, 2, 1 + k % 3) for k, i in enumerate(MIXED)]
    gss = [GpuScene(ctx, s) for s, _ in scenes]
    jobs = [BatchJob(g, s.camera_struct(), p) for g, (s, p) in zip(gss, scenes)]
    B = 1 << 14   # several wavefronts per job
    alone = []
    for g, (s, p) in zip(gss, scenes):
        r = PerPixelRenderer(g, s.camera_struct(), {"pt-x-samples": p.x_samples, "pt-y-samples": p.y_samples},
                             seed=p.seed, max_depth=p.max_depth, batch_paths=B)
        alone.append(r.render())
    for S in (1, 3, 8):
        films, ms, st = render_batch(ctx, jobs, streams=S, batch_paths=B)
        for f, a in zip(films, alone):
            # the same paths; only the order in which a vertex's shadow rays
            # (one per light) add into its radiance may differ (float atomics)
            assert np.allclose(f, a, rtol=1e-5, atol=1e-7), np.abs(f - a).max()
        assert st.streams == S and st.batch_paths == B
        assert st.paths == sum(s.camera["width"] ** 2 * p.x_samples * p.y_samples for s, p in scenes)
        assert st.extension_rays > st.paths and st.nonfinite == 0
        assert st.device_ms > 0 and st.wall_ms >= st.device_ms * 0.5
        assert (ms > 0).all()
        waves = sum(-(-(s.camera["width"] ** 2 * p.x_samples * p.y_samples) // B) for s, p in scenes)
        assert st.kernel_launches == sum(
            (2 + 3 * p.max_depth) * -(-(s.camera["width"] ** 2 * p.x_samples * p.y_samples) // B) + 1
            for s, p in scenes)
        assert waves > len(scenes)


@pytest.mark.gpu
def test_batch_jobs_match_oracle_path_by_path(ctx):
    from renderer_gb300.batch import BatchJob, render_batch
    scenes = [shrunk(i, 32, 2, 2, seed=11 + i) for i in SMALL]
    gss = [GpuScene(ctx, s) for s, _ in scenes]
    films, _, st = render_batch(ctx, [BatchJob(g, s.camera_struct(), p) for g, (s, p) in zip(gss, scenes)],
                                streams=2)
    for f, (s, p) in zip(films, scenes):
        o = OracleScene(s).render(s.camera_struct(), p, rng_mode=1)["film"].astype(np.float64)
        a = f.astype(np.float64)
        close = np.abs(a - o) <= 2e-3 * np.maximum(np.abs(o), 1e-3)
        assert close.all(-1).mean() >= 0.97
        assert a.sum() == pytest.approx(o.sum(), rel=2e-2)


@pytest.mark.gpu
def test_autotune_keeps_its_choice(ctx):
    from renderer_gb300.batch import BatchJob, autotune, render_batch
    scenes = [shrunk(i, 64, 1, 1) for i in SMALL]
    gss = [GpuScene(ctx, s) for s, _ in scenes]
    jobs = [BatchJob(g, s.camera_struct(), p) for g, (s, p) in zip(gss, scenes)]
    S, B = autotune(ctx, jobs)
    assert S in (1, 2, 4, 8) and B in (1 << 22, 1 << 24)
    _, _, st = render_batch(ctx, jobs)
    assert st.streams == S and st.batch_paths == B


@pytest.mark.gpu
def test_bad_jobs_are_refused(ctx):
    from renderer_gb300 import lib
    from renderer_gb300.batch import BatchJob, _jobs_array
    s, p = shrunk(9, 16, 1, 1)
    g = GpuScene(ctx, s)
    cam = s.camera_struct()
    arr = _jobs_array([BatchJob(g, cam, p)], None)   # no film
    st = _abi.BatchStats()
    assert lib().gbrt_render_batch(ctx.handle, arr, 1, 0, 0, None, C.byref(st)) == _abi.ERR_INVALID_ARG
    bad = render_params(1, 1, 1.5, 8, 0)             # termination probability outside [0, 1]
    from renderer_gb300.batch import render_batch
    with pytest.raises(GbrtError):
        render_batch(ctx, [BatchJob(g, cam, bad)])
    with pytest.raises(GbrtError):
        render_batch(ctx, [BatchJob(g, cam, p)], streams=65)
    # an empty batch is a no-op
    films, ms, st = render_batch(ctx, [])
    assert films == [] and st.paths == 0


# ------------------------------------------------- single-launch batch ----
def _alone(ctx, gss, scenes):
    """Each job rendered by itself through gbrt_render with its own params."""
    from renderer_gb300 import check, lib
    out = []
    for g, (s, p) in zip(gss, scenes):
        film = np.zeros((s.camera["height"], s.camera["width"], 3), np.float32)
        cam = s.camera_struct()
        check(lib().gbrt_render(g.handle, C.byref(cam), C.byref(p), film.ctypes.data_as(C.c_void_p), None, None,
                                None, None), ctx.handle)
        out.append(film)
    return out


@pytest.mark.gpu
def test_fused_batch_equals_individual_renders(ctx):
    """Wavefronts that cut through jobs and through pixels (B = 2^14 and an
    odd 10,007), and one wavefront for everything: every film equals the job
    rendered alone, up to the order of the FP64 pixel sums and of a vertex's
    shadow-ray additions."""
    from renderer_gb300.batch import BatchJob, render_batch_fused
    scenes = [shrunk(i, 48 + 16 * k, 2, 1 + k % 3) for k, i in enumerate(MIXED)]
    gss = [GpuScene(ctx, s) for s, _ in scenes]
    jobs = [BatchJob(g, s.camera_struct(), p) for g, (s, p) in zip(gss, scenes)]
    alone = _alone(ctx, gss, scenes)
    total = sum(s.camera["width"] ** 2 * p.x_samples * p.y_samples for s, p in scenes)
    D = max(p.max_depth for _, p in scenes)
    for B, P, tb, sb in ((1 << 14, 1, 128, 256), (10007, 3, 64, 128), (1 << 24, 2, 128, 128), (1 << 15, 4, 64, 256)):
        films, ms, st = render_batch_fused(ctx, jobs, wavefront_paths=B, pipelines=P, trace_block=tb, shade_block=sb)
        for f, a in zip(films, alone):
            assert np.allclose(f, a, rtol=1e-5, atol=1e-7), np.abs(f - a).max()
        waves = -(-total // min(B, total))
        assert st.streams == min(P, waves) and st.batch_paths == min(B, total) and st.paths == total
        assert st.kernel_launches == waves * (4 + 3 * D) + 1
        assert st.extension_rays > st.paths and st.nonfinite == 0
        # the last job ends with the last wavefront; the batch's span also
        # takes the join of the pipelines' streams
        assert (ms > 0).all() and 0.9 * st.device_ms <= ms.max() <= st.device_ms * 1.001 + 0.01


@pytest.mark.gpu
def test_fused_batch_physical_with_instances_and_textures(ctx):
    """The general traversal (mesh instances) and the texture shading in one
    batch with plain scenes, under the physical estimator."""
    from renderer_gb300.batch import BatchJob, render_batch_fused
    from tests.test_instances import instanced_cornell
    from tests.test_texture import textured_room
    si, _ = instanced_cornell(40, smooth=False)
    st_ = textured_room()
    st_.camera["width"] = st_.camera["height"] = 40
    plain, _ = shrunk(9, 48, 1, 1)
    prm = [render_params(2, 2, 0.5, 8, 21, semantics=_abi.SEM_PHYSICAL),
           render_params(1, 2, 0.5, 6, 22, semantics=_abi.SEM_PHYSICAL),
           render_params(2, 1, 0.5, 5, 23, semantics=_abi.SEM_PHYSICAL)]
    scenes = list(zip((si, st_, plain), prm))
    gss = [GpuScene(ctx, s) for s, _ in scenes]
    jobs = [BatchJob(g, s.camera_struct(), p) for g, (s, p) in zip(gss, scenes)]
    alone = _alone(ctx, gss, scenes)
    films, _, st = render_batch_fused(ctx, jobs, wavefront_paths=5000, pipelines=2)
    for f, a in zip(films, alone):
        assert np.allclose(f, a, rtol=1e-5, atol=1e-7), np.abs(f - a).max()
    # and against the oracle, path by path
    for f, (s, p) in zip(films, scenes):
        o = OracleScene(s).render(s.camera_struct(), p, rng_mode=1)["film"].astype(np.float64)
        close = np.abs(f - o) <= 2e-3 * np.maximum(np.abs(o), 1e-3)
        assert close.all(-1).mean() >= 0.95


@pytest.mark.gpu
def test_fused_autotune_and_refusals(ctx):
    from renderer_gb300 import lib
    from renderer_gb300.batch import BatchJob, _jobs_array, autotune_fused, render_batch_fused
    scenes = [shrunk(i, 64, 1, 1) for i in SMALL]
    gss = [GpuScene(ctx, s) for s, _ in scenes]
    jobs = [BatchJob(g, s.camera_struct(), p) for g, (s, p) in zip(gss, scenes)]
    c = autotune_fused(ctx, jobs)
    assert c["wavefront_paths"] in (1 << 20, 1 << 22, 1 << 24) and c["pipelines"] in (1, 2, 4)
    assert c["trace_block"] in (64, 128) and c["shade_block"] in (128, 256)
    assert c["pipelines"] * c["wavefront_paths"] <= 1 << 25
    _, _, st = render_batch_fused(ctx, jobs)
    total = sum(s.camera["width"] ** 2 for s, _ in scenes)
    assert st.batch_paths == min(c["wavefront_paths"], total)
    # one estimator for all jobs
    mixed = [jobs[0], BatchJob(gss[1], jobs[1].camera, render_params(1, 1, 0.5, 8, 0, semantics=_abi.SEM_PHYSICAL))]
    with pytest.raises(GbrtError):
        render_batch_fused(ctx, mixed)
    with pytest.raises(GbrtError):
        render_batch_fused(ctx, jobs, trace_block=96)
    arr = _jobs_array(jobs[:1], None)  # no film
    s = _abi.BatchStats()
    assert lib().gbrt_render_batch_fused(ctx.handle, arr, 1, None, None, C.byref(s)) == _abi.ERR_INVALID_ARG
    with pytest.raises(GbrtError):
        render_batch_fused(ctx, jobs, pipelines=9)
    films, ms, st = render_batch_fused(ctx, [])
    assert films == [] and st.paths == 0


@pytest.mark.gpu
def test_fused_batch_extreme_wavefronts(ctx):
    """Wavefronts of a single path (every graph replay shades one path of one
    job) and of three paths, with 1 x 1 and 5 x 3 images among larger ones:
    the films still equal the jobs rendered alone."""
    from renderer_gb300.batch import BatchJob, render_batch_fused
    scenes = [shrunk(9, 1, 1, 1), shrunk(6, 5, 2, 1), shrunk(8, 12, 1, 2)]
    scenes[1][0].camera["height"] = 3
    gss = [GpuScene(ctx, s) for s, _ in scenes]
    jobs = [BatchJob(g, s.camera_struct(), p) for g, (s, p) in zip(gss, scenes)]
    alone = _alone(ctx, gss, scenes)
    total = sum(s.camera["width"] * s.camera["height"] * p.x_samples * p.y_samples for s, p in scenes)
    for B, P in ((1, 1), (3, 2)):
        films, ms, st = render_batch_fused(ctx, jobs, wavefront_paths=B, pipelines=P)
        assert st.paths == total and st.batch_paths == B
        for f, a in zip(films, alone):
            assert f.shape == a.shape
            assert np.allclose(f, a, rtol=1e-5, atol=1e-7), np.abs(f - a).max()
