"""The checked build (renderer_gb300/build.py, build(checked=True)): the same
kernels compiled with -DGBRT_CHECKED test every index they follow (tree nodes,
leaf records, instances, hit records, lights, materials, queue slots) and
report a failure in the call's status instead of reading or writing outside a
buffer. This is the sanitizer of this project's device code (compute-sanitizer
is closed on the GPU pool).

The test builds the checked library, renders the same set of scenes with both
libraries in child processes (one CUDA library per process), and requires
every call to succeed and the images to agree: plain, textured, CSG and
instanced scenes under both estimators, a guided render, a Metropolis render,
ray queries and a single-launch batch."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import os, sys
sys.path.insert(0, os.environ["GBRT_ROOT"])
import numpy as np
import renderer_gb300
renderer_gb300.LIB_PATH = sys.argv[1]
from renderer_gb300 import GpuScene, PerPixelRenderer, _abi, check, lib, workloads
from renderer_gb300.runtime import Context, make_rays
from renderer_gb300.scene import render_params
from tests.test_csg import csg_scene
from tests.test_instances import instanced_cornell
from tests.test_texture import textured_room
out = {}
with Context(0) as ctx:
    def render(s, p):
        import ctypes as C
        film = np.zeros((s.camera["height"], s.camera["width"], 3), np.float32)
        cam = s.camera_struct()
        g = GpuScene(ctx, s)
        check(lib().gbrt_render(g.handle, C.byref(cam), C.byref(p), film.ctypes.data_as(C.c_void_p), None, None,
                                None, None), ctx.handle)
        return film, g
    scenes = {"cornell": workloads.cornell_box(48, 48), "csg": csg_scene(), "instanced": instanced_cornell(40)[0],
              "textured": textured_room()}
    for name, s in scenes.items():
        for sem in (_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL):
            f, g = render(s, render_params(2, 2, 0.5, 8, 3, semantics=sem))
            out["%s_%d" % (name, sem)] = f
    rng = np.random.default_rng(0)
    g = GpuScene(ctx, scenes["instanced"])
    rays = make_rays(rng.uniform(-0.9, 0.9, (20000, 3)) + [0, 1, 0], rng.normal(size=(20000, 3)))
    out["trace_prim"] = g.intersect(rays)["prim"].astype(np.float64)
    from renderer_gb300.chains import MetropolisRenderer
    m = MetropolisRenderer(GpuScene(ctx, scenes["cornell"]), options={"met-mutations": 4, "met-bootstrap": 500},
                           seed=2, chains=64)
    out["mlt"] = m.render()
    from renderer_gb300.guiding import Guide, guide_params, render_guided, scene_bounds
    gr = GpuScene(ctx, scenes["cornell"])
    guide = Guide(ctx, scene_bounds(gr), seed=1)
    gcam = scenes["cornell"].camera_struct()
    gpar = render_params(1, 1, 0.5, 8, 5, semantics=_abi.SEM_PHYSICAL)
    film, st = render_guided(gr, gcam, gpar, guide,
                             guide_params(0.5, passes=4, train_passes=4, steps_per_pass=2, batch_samples=1 << 14))
    out["guided_mean"] = np.array([film.mean()])
    # a fixed network (no training): inference and guided shading are deterministic
    guide.set_weights(np.random.default_rng(3).normal(0.0, 0.1, _abi.GUIDE_PARAMS).astype(np.float32))
    out["guided_fixed"], _ = render_guided(gr, gcam, gpar, guide, guide_params(0.5, passes=2))
    guide.close()
    from renderer_gb300.batch import BatchJob, render_batch_fused
    jobs = [BatchJob(GpuScene(ctx, scenes[k]), scenes[k].camera_struct(), render_params(2, 1, 0.5, 6, 9))
            for k in ("cornell", "textured")]
    films, _, _ = render_batch_fused(ctx, jobs, wavefront_paths=4000, pipelines=2)
    out["batch0"], out["batch1"] = films
np.savez(sys.argv[2], **out)
print("ok", len(out))
'''


def _run(lib_path, out_path):
    env = dict(os.environ, GBRT_ROOT=ROOT)
    r = subprocess.run([sys.executable, "-c", CHILD, lib_path, str(out_path)], capture_output=True, text=True,
                       env=env, cwd=ROOT, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    return np.load(out_path)


def test_checked_build_renders_the_same_images(tmp_path):
    from renderer_gb300 import LIB_PATH, build
    checked = build.build(checked=True)
    assert checked != LIB_PATH and os.path.exists(checked)
    a = _run(checked, tmp_path / "checked.npz")
    b = _run(LIB_PATH, tmp_path / "normal.npz")
    assert set(a.files) == set(b.files) and len(a.files) >= 12
    for k in a.files:
        if k == "guided_mean":
            # training gathers gradients with float atomics, so the two guides
            # differ in their last bits and the guided paths part ways: the
            # images are two estimates of one mean (4 spp of a 48 x 48 box)
            assert a[k][0] == pytest.approx(b[k][0], rel=0.2)
        elif k == "trace_prim":
            assert np.array_equal(a[k], b[k])
        else:
            assert np.allclose(a[k], b[k], rtol=1e-5, atol=1e-6), (k, np.abs(a[k] - b[k]).max())
