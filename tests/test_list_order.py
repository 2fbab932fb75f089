"""Exact ties in t under GBRT_SCENE_LIST_ORDER: the renderer's IntersectableList
rule (src/intersectablelist.cpp:29-47, the root the renderer traverses with
--no-bvh, src/sceneast.cpp:681-688): each entry is tested with the ray
shortened to the best hit so far, inclusive, so of two hits at the same t the
later entry in the list wins.

The tie scene duplicates geometry with different materials: identical
triangles, a triangle equal to a quad's first half, identical spheres,
identical planes, duplicated triangles inside a mesh and two instances of that
mesh under one transform. Every duplicate pair gives bit-identical t, so the
winner is decided by the tie rule alone. The oracle with use_bvh=False is the
renderer's list; the GPU traverses its BVH with the flag.

CPU: the parser's list ranks follow the scene file; the oracle's winner follows
the ranks. GPU: the same primitive as the oracle on every ray, and path-level
parity of a render whose colours show which duplicate won."""
import numpy as np
import pytest

from oracle.binding import OracleScene
from renderer_gb300 import _abi
from renderer_gb300.runtime import make_rays
from renderer_gb300.scene import SceneData, render_params

COLOURS = [(0.9, 0.1, 0.1), (0.1, 0.9, 0.1), (0.1, 0.1, 0.9), (0.8, 0.8, 0.1), (0.1, 0.8, 0.8), (0.8, 0.1, 0.8)]


def tie_scene(seed=0, width=48):
    rng = np.random.default_rng(seed)
    s = SceneData()
    mats = [s.add_material(_abi.MAT_DIFFUSE, kd=c) for c in COLOURS]
    # left third of the floor: two identical triangles, and a triangle equal
    # to the first half of a quad (Quad(p1..p4) = Tri(p1,p2,p4) + Tri(p4,p2,p3))
    p1, p2, p3, p4 = (-1, 0, -1), (-0.34, 0, -1), (-0.34, 0, 1), (-1, 0, 1)
    tri = np.array(p1 + p2 + p4, np.float32)
    tris = [tri, tri, np.array(p4 + p2 + p3, np.float32)]
    s.tri_pos = np.array(tris, np.float32)
    s.tri_mat = np.array([mats[0], mats[1], mats[2]], np.int32)
    s.quads = [(p1, p2, p3, p4, mats[3])]
    # middle: three identical spheres
    s.spheres = [((0.0, 0.2, 0.0), 0.3, mats[k]) for k in (4, 5, 0)]
    # below everything: two identical planes y = -0.5
    s.planes = [((0, 1, 0, 0.5), mats[1]), ((0, 1, 0, 0.5), mats[2])]
    # right third: a relief mesh holding every triangle twice (different
    # materials), instanced twice under the same transform
    n = 6
    xs = np.linspace(0, 1, n + 1)
    h = 0.1 * rng.random((n + 1, n + 1))
    mt, mm = [], []
    for i in range(n):
        for j in range(n):
            a = (xs[i], h[i, j], xs[j]); b = (xs[i + 1], h[i + 1, j], xs[j])
            c = (xs[i + 1], h[i + 1, j + 1], xs[j + 1]); d = (xs[i], h[i, j + 1], xs[j + 1])
            for q in ((a, b, c), (a, c, d)):
                for copy in (0, 1):
                    mt.append(np.array(q, np.float32).reshape(-1))
                    mm.append(mats[(2 * copy + i + j) % len(mats)])
    m = s.add_mesh(np.array(mt), mat=np.array(mm, np.int32))
    T = np.array([[0.6, 0, 0, 0.38], [0, 0.6, 0, 0.0], [0, 0, 1.8, -0.9]], np.float32)
    s.add_instance(T, m)
    s.add_instance(T, m)
    s.lights = [dict(type=_abi.LIGHT_POINT, origin=(0.1, 2.5, 0.3), intensity=(6, 6, 6))]
    s.camera = dict(eye=(0, 3, 0.001), look_at=(0, 0, 0), up=(0, 0, -1), fov=0.9, width=width, height=width)
    s.list_rank = rng.permutation(s.n_prims()).astype(np.int32)
    s.flags = _abi.SCENE_LIST_ORDER
    return s


def down_rays(n, seed=1):
    rng = np.random.default_rng(seed)
    o = np.stack([rng.uniform(-1.1, 1.1, n), np.full(n, 2.0), rng.uniform(-1.1, 1.1, n)], -1)
    d = np.stack([rng.normal(0, 0.05, n), -np.ones(n), rng.normal(0, 0.05, n)], -1)
    return make_rays(o, d)


def test_parser_ranks_follow_the_file(tmp_path):
    """Lights first, then the intersectables as listed, whatever their kind."""
    from renderer_gb300.scenefile import load_scene_string
    s = load_scene_string("""
        lights = lights { pointlight([0 2 0], [1 1 1]) };
        m = diffuse([0.5 0.5 0.5]);
        intersectable = intersectables {
          sphere([0 0 0], 1, m)
          t([0 0 0], [1 0 0], [0 1 0], [0 0 0], [0 0 0], [0 0 0], [0 0], [0 0], [0 0], m)
          plane([0 1 0 0], m)
          intersectables { quad([0 0 0], [1 0 0], [1 1 0], [0 1 0], m) sphere([2 0 0], 1, m) }
          t([0 0 1], [1 0 1], [0 1 1], [0 0 0], [0 0 0], [0 0 0], [0 0], [0 0], [0 0], m)
        };""")
    o = s.prim_offsets()
    want = {0: 0, o["spheres"]: 1, o["tri"]: 2, o["planes"]: 3, o["quads"]: 4, o["spheres"] + 1: 5, o["tri"] + 1: 6}
    assert s.list_rank is not None and len(s.list_rank) == s.n_prims() == 7
    for pid, r in want.items():
        assert s.list_rank[pid] == r, (pid, s.list_rank)


def test_oracle_list_takes_the_later_entry():
    """The oracle's list mode: of the duplicates the highest-ranked one wins;
    reversing the ranks changes the winner wherever two duplicates tie."""
    s = tie_scene()
    rays = down_rays(20000)
    h = OracleScene(s, use_bvh=False).intersect(rays)
    o = s.prim_offsets()
    tri_hit = (h["prim"] >= o["tri"]) & (h["prim"] < o["spheres"])
    # the first-half triangle region: one of tri 0 / tri 1 / the quad
    cands = np.array([o["tri"], o["tri"] + 1, o["quads"]])
    best = cands[np.argmax(s.list_rank[cands])]
    # hits well inside Tri(p1, p2, p4): x in [-1, -0.34], z from -1 up to the p2-p4 diagonal
    p = rays["org"] + h["t"][:, None] * rays["dir"]
    u, w = (p[:, 0] + 1) / 0.66, (p[:, 2] + 1) / 2
    region = np.isfinite(h["t"]) & (u > 0.02) & (w > 0.02) & (u + w < 0.98)
    assert tri_hit.any()
    sel = region & np.isin(h["prim"], cands)
    assert sel.sum() > 100
    assert np.all(h["prim"][sel] == best)
    r = s.list_rank.copy()
    s.list_rank = (r.max() - r).astype(np.int32)
    h2 = OracleScene(s, use_bvh=False).intersect(rays)
    changed = (h2["prim"] != h["prim"]) & np.isfinite(h["t"])
    assert changed.sum() > 1000
    assert np.array_equal(h2["t"][changed], h["t"][changed])  # same t: only the tie rule changed


@pytest.mark.gpu
def test_gpu_list_order_ray_by_ray(ctx):
    from renderer_gb300 import GpuScene
    for seed in (0, 1, 2):
        s = tie_scene(seed)
        rays = down_rays(100000, seed + 10)
        g = GpuScene(ctx, s).intersect(rays)
        o = OracleScene(s, use_bvh=False).intersect(rays)
        same = g["prim"] == o["prim"]
        # identical t, and no tie decided the other way
        tie_flip = ~same & (g["t"] == o["t"])
        assert not tie_flip.any(), (seed, np.nonzero(tie_flip)[0][:10])
        assert same.mean() >= 0.99999, same.mean()
        both = same & np.isfinite(o["t"])
        assert np.array_equal(g["t"][both], o["t"][both])


@pytest.mark.gpu
@pytest.mark.parametrize("semantics", [_abi.SEM_REFERENCE, _abi.SEM_PHYSICAL])
def test_gpu_list_order_render_path_by_path(ctx, semantics):
    """The colours of the winning duplicates (mesh-internal and cross-instance
    ties included), path by path against the oracle's list."""
    from tests.test_gpu_render import gpu_render
    s = tie_scene(3, width=40)
    prm = render_params(2, 2, 0.5, 3, 4, semantics=semantics)
    (film, _, _), _ = gpu_render(ctx, s, prm)
    orc = OracleScene(s, use_bvh=False).render(s.camera_struct(), prm, rng_mode=1)["film"]
    close = np.isclose(film, orc, rtol=2e-3, atol=1e-5).all(-1)
    assert close.mean() > 0.98, close.mean()
    # and the flag matters: the reversed ranks give another image
    s.list_rank = (s.list_rank.max() - s.list_rank).astype(np.int32)
    (film2, _, _), _ = gpu_render(ctx, s, prm)
    orc2 = OracleScene(s, use_bvh=False).render(s.camera_struct(), prm, rng_mode=1)["film"]
    assert np.isclose(film2, orc2, rtol=2e-3, atol=1e-5).all(-1).mean() > 0.98
    assert np.abs(film2 - film).max() > 0.05
