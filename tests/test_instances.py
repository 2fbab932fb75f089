"""Instanced meshes and the two-level BVH (gbrt_mesh, gbrt_instance;
IntersectableInstance, src/intersectableinstance.cpp:24-46).

CPU: in the oracle, an instance hits where its mesh transformed into world
space hits (same t, the instance's prim id, the same normal). GPU: closest-hit
and any-hit queries equal the oracle's ray by ray; renders match the oracle
path by path under both estimators; the two-level scene renders the image of
the flattened one; the ABI refuses bad instance tables."""
import ctypes as C

import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import GbrtError, GpuScene, PerPixelRenderer, _abi, workloads
from renderer_gb300.runtime import make_rays
from renderer_gb300.scene import SceneData, render_params


def rot(axis, deg):
    a = np.radians(deg)
    c, s = np.cos(a), np.sin(a)
    x, y, z = np.asarray(axis, float) / np.linalg.norm(axis)
    return np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                     [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                     [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])


def xform(R, t, scale=1.0):
    M = np.zeros((3, 4))
    M[:, :3] = R * scale
    M[:, 3] = t
    return M


TRANSFORMS = [xform(rot((0, 1, 0), 0), (-0.55, 0.45, -0.4), 0.6),
              xform(rot((0, 1, 0), 40), (0.5, 0.55, -0.3), 0.5),
              xform(rot((1, 0.3, 0), 75), (-0.3, 1.2, 0.3), 0.45),
              xform(rot((0.2, 1, 0.5), 130), (0.45, 1.3, 0.35), 0.55)]


def relief(n=24, seed=3):
    """A noise-displaced heightfield patch over [-1, 1]^2 (z up to -0.3)."""
    return workloads.displaced_grid(n, -1.0, 1.0, -1.0, 1.0, 0.0, 0.3, seed)


def instanced_cornell(width=48, transforms=TRANSFORMS, smooth=True):
    """The Cornell room with a relief mesh placed by each transform (two
    materials), and its flattened twin."""
    s = workloads.cornell_box(width, width)
    pos, nrm = relief()
    glossy = s.add_material(_abi.MAT_BLINN, kd=(0.3, 0.25, 0.2), ks=(0.4, 0.4, 0.4), exponent=40.0)
    diffuse = 0
    mat = np.where(np.arange(len(pos)) % 3 == 0, glossy, diffuse).astype(np.int32)
    mi = s.add_mesh(pos, nrm if smooth else None, mat)
    for M in transforms:
        s.add_instance(M, mi)
    f = workloads.cornell_box(width, width)
    f.add_material(_abi.MAT_BLINN, kd=(0.3, 0.25, 0.2), ks=(0.4, 0.4, 0.4), exponent=40.0)
    P, N, MM = [], [], []
    for M in transforms:
        A = M[:, :3].astype(np.float32)
        t = M[:, 3].astype(np.float32)
        P.append((pos.reshape(-1, 3) @ A.T + t).reshape(-1, 9))
        nn = nrm.reshape(-1, 3) @ np.linalg.inv(A.astype(np.float64))
        N.append((nn / np.linalg.norm(nn, axis=1, keepdims=True)).reshape(-1, 9))
        MM.append(mat)
    f.tri_pos = np.concatenate(P).astype(np.float32)
    f.tri_nrm = np.concatenate(N).astype(np.float32) if smooth else None
    f.tri_mat = np.concatenate(MM)
    return s, f


def random_rays(n, seed=0):
    rng = np.random.default_rng(seed)
    org = np.column_stack([rng.uniform(-0.9, 0.9, n), rng.uniform(0.1, 1.9, n), rng.uniform(-0.9, 2.5, n)])
    d = rng.normal(size=(n, 3))
    return make_rays(org, d / np.linalg.norm(d, axis=1, keepdims=True))


def test_oracle_instance_equals_transformed_mesh():
    s, f = instanced_cornell()
    rays = random_rays(20000, 1)
    hi = OracleScene(s).intersect(rays)
    hf = OracleScene(f).intersect(rays)
    off_s, off_f = s.prim_offsets(), f.prim_offsets()
    ntri = len(relief()[0])
    inst_s = (hi["prim"] >= off_s["instances"])
    tri_f = (hf["prim"] >= off_f["tri"]) & (hf["prim"] < off_f["tri"] + f.n_tri())
    assert inst_s.sum() > 2000
    agree = np.mean(inst_s == tri_f)
    assert agree > 0.999
    both = inst_s & tri_f
    # the instance hit by a ray is the one whose copy the flattened scene hits
    assert np.mean((hi["prim"][both] - off_s["instances"]) == (hf["prim"][both] - off_f["tri"]) // ntri) > 0.999
    assert np.allclose(hi["t"][both], hf["t"][both], rtol=1e-4, atol=1e-6)
    other = ~inst_s & ~tri_f
    pf = hf["prim"][other]
    pf = np.where(pf >= off_f["quads"], pf - f.n_tri(), pf)  # the flattened twin numbers its triangles first
    assert np.array_equal(hi["prim"][other], pf)


@pytest.mark.gpu
def test_gpu_instances_match_oracle_ray_by_ray(ctx):
    s, _ = instanced_cornell()
    rays = random_rays(200000, 2)
    g = GpuScene(ctx, s).intersect(rays)
    o = OracleScene(s).intersect(rays)
    same = g["prim"] == o["prim"]
    assert same.mean() > 0.9999
    hit = same & np.isfinite(o["t"])
    assert np.allclose(g["t"][hit], o["t"][hit], rtol=1e-5, atol=1e-7)
    inst = hit & (o["prim"] >= s.prim_offsets()["instances"])
    assert inst.sum() > 20000
    assert np.allclose(g["u"][inst], o["u"][inst], atol=1e-4)


@pytest.mark.gpu
def test_gpu_instances_any_hit(ctx):
    s, _ = instanced_cornell()
    rays = random_rays(100000, 3)
    rays["tmax"] = np.float32(1.0)
    gs = GpuScene(ctx, s)
    g = gs.occluded(rays)
    o = OracleScene(s).occluded(rays)
    assert np.mean(g == o) > 0.9999
    assert 0.1 < g.mean() < 0.95


def _path_level(ctx, s, params, min_frac=0.97):
    film = PerPixelRenderer(GpuScene(ctx, s), s.camera_struct(),
                            {"pt-x-samples": params.x_samples, "pt-y-samples": params.y_samples,
                             "pt-termination-prob": params.termination_prob},
                            seed=params.seed, max_depth=params.max_depth).render() \
        if params.semantics == _abi.SEM_REFERENCE else None
    if film is None:
        from renderer_gb300 import check, lib
        film = np.zeros((s.camera["height"], s.camera["width"], 3), np.float32)
        st = _abi.Stats()
        gs = GpuScene(ctx, s)
        cam = s.camera_struct()
        check(lib().gbrt_render(gs.handle, C.byref(cam), C.byref(params), film.ctypes.data_as(C.c_void_p), None,
                                None, None, C.byref(st)), ctx.handle)
    o = OracleScene(s).render(s.camera_struct(), params, rng_mode=1)["film"]
    a, b = film.astype(np.float64), o.astype(np.float64)
    close = (np.abs(a - b) <= 2e-3 * np.maximum(np.abs(b), 1e-3)).all(-1).mean()
    assert close >= min_frac, close
    assert a.sum() == pytest.approx(b.sum(), rel=1e-2)


@pytest.mark.gpu
def test_gpu_instanced_render_matches_oracle_path_by_path(ctx):
    s, _ = instanced_cornell(48)
    _path_level(ctx, s, render_params(2, 2, 0.5, 8, 5))


@pytest.mark.gpu
def test_gpu_instanced_render_physical_matches_oracle(ctx):
    s, _ = instanced_cornell(40, smooth=False)
    _path_level(ctx, s, render_params(2, 2, 0.5, 8, 6, semantics=_abi.SEM_PHYSICAL), min_frac=0.95)


@pytest.mark.gpu
def test_two_level_renders_the_flattened_image(ctx):
    s, f = instanced_cornell(64)
    opts = {"pt-x-samples": 8, "pt-y-samples": 8}
    a = PerPixelRenderer(GpuScene(ctx, s), options=opts, seed=1, max_depth=6).render()
    b = PerPixelRenderer(GpuScene(ctx, f), options=opts, seed=2, max_depth=6).render()
    assert a.mean() == pytest.approx(b.mean(), rel=0.02)
    blk = lambda x: x.mean(-1).reshape(8, 8, 8, 8).mean((1, 3))  # noqa: E731
    assert np.median(np.abs(blk(a) - blk(b)) / np.maximum(blk(b), 1e-3)) < 0.05


@pytest.mark.gpu
def test_bad_instance_tables_are_refused(ctx):
    s, _ = instanced_cornell(8)
    s.instances[1] = (np.zeros((3, 4), np.float32), 0)  # singular
    with pytest.raises(GbrtError):
        GpuScene(ctx, s)
    s, _ = instanced_cornell(8)
    s.instances[0] = (s.instances[0][0], 5)  # no such mesh
    with pytest.raises(GbrtError):
        GpuScene(ctx, s)
