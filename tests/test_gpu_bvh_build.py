"""The GPU BVH builder (GBRT_SCENE_GPU_BUILD): a linear BVH over Morton codes
collapsed to the traversal's 4-wide nodes. The tree differs from the host's
SAH tree, the hits must not: ray-level parity with the oracle's
BVHNode::intersect at the same bar as the host-built tree, identical renders
(same random numbers, the same hits) and small, degenerate and duplicate-box
scenes."""
import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import GpuScene, _abi, workloads
from renderer_gb300.scene import SceneData
from tests.test_gpu_trace import box_rays, compare, run_parity

pytestmark = pytest.mark.gpu


def gpu_built(s):
    s.flags = _abi.SCENE_GPU_BUILD
    return s


def test_gpu_build_parity_cornell_box(ctx):
    rng = np.random.default_rng(10)
    gs, _, _, _ = run_parity(ctx, gpu_built(workloads.cornell_box(128, 128)), rng, n_per_pixel=2)
    info = gs.info()
    assert info["max_depth"] == 0 and info["nodes"] >= 1


def test_gpu_build_parity_icosphere(ctx):
    rng = np.random.default_rng(11)
    s = gpu_built(workloads.icosphere_scene(levels=6, width=256, height=256, env_size=(64, 32)))
    gs, _, _, _ = run_parity(ctx, s, rng, n_per_pixel=2)
    assert gs.info()["leaves"] > 0


def test_gpu_build_parity_full_mesh(ctx):
    """1,310,720 triangles: the scale the builder is for."""
    rng = np.random.default_rng(12)
    s = gpu_built(workloads.icosphere_scene(levels=8, width=384, height=384, env_size=(64, 32)))
    gs, _, _, _ = run_parity(ctx, s, rng, n_box=100000, n_per_pixel=1)
    host = GpuScene(ctx, workloads.icosphere_scene(levels=8, width=8, height=8, env_size=(64, 32)))
    # a few milliseconds on the device against the host's seconds
    assert gs.info()["build_ms"] < host.info()["build_ms"]


@pytest.mark.parametrize("n", [1, 2, 7, 8, 9, 100, 4099])
def test_gpu_build_small_and_ragged(ctx, n):
    """Scenes of a handful of primitives (one leaf, a root with few children)
    and sizes around the sort's tile."""
    rng = np.random.default_rng(n)
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.5, 0.5, 0.5))
    c = rng.uniform(-1, 1, (n, 3))
    tri = np.concatenate([c, c + rng.uniform(-0.1, 0.1, (n, 3)), c + rng.uniform(-0.1, 0.1, (n, 3))], 1)
    s.tri_pos = tri.astype(np.float32)
    s.tri_mat = np.full(n, m, np.int32)
    s.camera = dict(eye=(0, 0, 3), look_at=(0, 0, 0), up=(0, 1, 0), fov=0.8, width=8, height=8)
    orc = OracleScene(s)
    gs = GpuScene(ctx, gpu_built(s))
    rays = box_rays(s, rng, 20000)
    compare(gs.intersect(rays), orc.intersect(rays, threads=0), "n=%d" % n)


def test_gpu_build_duplicate_boxes(ctx):
    """Many primitives with the same Morton code (equal centres): the index
    tie-break keeps the tree well formed."""
    rng = np.random.default_rng(3)
    n = 5000
    s = SceneData()
    m = s.add_material(_abi.MAT_DIFFUSE, kd=(0.5, 0.5, 0.5))
    base = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float64)
    tri = np.repeat(base, n, 0) + rng.normal(0, 1e-7, (n, 9))
    tri[:10] += rng.uniform(-2, 2, (10, 9))
    s.tri_pos = tri.astype(np.float32)
    s.tri_mat = np.full(n, m, np.int32)
    s.camera = dict(eye=(0.3, 0.3, 3), look_at=(0.3, 0.3, 0), up=(0, 1, 0), fov=0.5, width=8, height=8)
    orc = OracleScene(s)
    gs = GpuScene(ctx, gpu_built(s))
    rays = box_rays(s, rng, 20000)
    # thousands of coincident triangles: disagreements are exact-t ties,
    # which compare() requires of every mismatch
    compare(gs.intersect(rays), orc.intersect(rays, threads=0), "duplicates", min_frac=0.99)


def test_gpu_build_render_matches_host_build(ctx):
    """Same scene, same random numbers: the two trees give the same image (up
    to exact-t ties, absent here)."""
    from renderer_gb300.runtime import PerPixelRenderer
    s = workloads.cornell_box(64, 64)
    a = PerPixelRenderer(GpuScene(ctx, s), None, {"pt-x-samples": 2, "pt-y-samples": 2}, seed=5, max_depth=8)
    b = PerPixelRenderer(GpuScene(ctx, gpu_built(workloads.cornell_box(64, 64))), None,
                         {"pt-x-samples": 2, "pt-y-samples": 2}, seed=5, max_depth=8)
    fa, fb = a.render(), b.render()
    assert np.mean(np.isclose(fa, fb, rtol=1e-5, atol=1e-7)) > 0.999
