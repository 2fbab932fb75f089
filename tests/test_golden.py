"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py).

CPU: the library's Radiance reader decodes scanlines of the renderer's own
shipped light probe exactly as an independent numpy restatement of the
format does, and the oracle still reproduces its committed ray hits, its
Cornell-box images (reference and physically based estimators) and its
Metropolis image bit for bit. GPU: the CUDA traversal and path tracer are
held against the same fixtures, so the comparison does not depend on the
oracle being built where the GPU runs."""
import os

import numpy as np
import pytest

from renderer_gb300 import workloads

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_reader_decodes_probe_scanlines_like_the_restatement(gbrt_built):
    from renderer_gb300.scenefile import read_hdr
    z = _load("probe_rows.npz")
    img = read_hdr(os.path.join(GOLDEN, "probe_rows.hdr"))
    assert img.shape == z["texels"].shape == (8, 640, 3)
    assert np.array_equal(img, z["texels"])
    # the middle rows of the probe's disc, which reaches the image's edges
    assert np.all(np.isfinite(img)) and img.min() > 0
    assert tuple(z["full_shape"]) == (640, 640, 3)


def test_reader_matches_the_whole_probe_sums(reference_probe):
    from renderer_gb300.scenefile import read_hdr
    z = _load("probe_rows.npz")
    img = read_hdr(reference_probe)
    assert np.array_equal(img.astype(np.float64).sum((0, 1)), z["full_sums"])
    assert np.array_equal(img[316:324], z["texels"])


def test_oracle_reproduces_ray_fixture():
    from oracle.binding import OracleScene
    z = _load("cornell_rays.npz")
    hits = OracleScene(workloads.cornell_box(64, 64)).intersect(z["rays"])
    ref = z["hits"]
    assert np.array_equal(hits["prim"], ref["prim"])
    assert np.array_equal(hits["t"], ref["t"], equal_nan=True)
    # both camera and interior rays hit something; some rays from inside
    # the open box leave through its open side
    assert (ref["prim"][:2048] >= 0).mean() > 0.9 and (ref["prim"] == -1).any()


def test_oracle_reproduces_render_fixture():
    from oracle.binding import OracleScene
    z = _load("cornell_render.npz")
    s = workloads.cornell_box(32, 32)
    out = OracleScene(s).render(s.camera_struct(), workloads.cornell_params(max_depth=8, seed=7, x_samples=2,
                                                                            y_samples=2), rng_mode=1)
    assert np.array_equal(out["film"], z["film"])
    assert out["paths"] == int(z["paths"]) == 32 * 32 * 4



def test_oracle_reproduces_physical_and_metropolis_fixtures():
    from oracle.binding import OracleScene
    from renderer_gb300 import _abi
    from renderer_gb300.chains import mlt_params
    from renderer_gb300.scene import render_params
    z = _load("cornell_physical_mlt.npz")
    s = workloads.cornell_box(32, 32)
    phys = OracleScene(s).render(s.camera_struct(), render_params(2, 2, 0.5, 8, 9, semantics=_abi.SEM_PHYSICAL),
                                 rng_mode=1)
    assert np.array_equal(phys["film"], z["phys_film"])
    mlt = OracleScene(s).render_mlt(s.camera_struct(), render_params(1, 1, 0.0, 5, 2), mlt_params(8, 500), chains=64)
    assert np.array_equal(mlt["film"], z["mlt_film"])
    assert mlt["b"] == float(z["mlt_b"]) and mlt["accepted"] == int(z["mlt_accepted"])
    assert mlt["mutations"] == int(z["mlt_mutations"]) == 32 * 32 * 8  # met-mutations per pixel

@pytest.mark.gpu
def test_gpu_trace_matches_ray_fixture(ctx):
    from renderer_gb300 import GpuScene
    z = _load("cornell_rays.npz")
    g = GpuScene(ctx, workloads.cornell_box(64, 64)).intersect(z["rays"])
    ref = z["hits"]
    assert np.array_equal(g["prim"], ref["prim"])
    hit = ref["prim"] >= 0
    assert np.array_equal(g["t"][hit], ref["t"][hit])


@pytest.mark.gpu
def test_gpu_render_matches_render_fixture(ctx):
    from renderer_gb300 import GpuScene, PerPixelRenderer
    z = _load("cornell_render.npz")
    s = workloads.cornell_box(32, 32)
    r = PerPixelRenderer(GpuScene(ctx, s), s.camera_struct())
    r.params = workloads.cornell_params(max_depth=8, seed=7, x_samples=2, y_samples=2)
    film, _, _ = r.render(want_moments=True)
    a, b = film.astype(np.float64), z["film"].astype(np.float64)
    close = np.abs(a - b) <= 2e-3 * np.maximum(np.abs(b), 1e-3)
    assert close.all(-1).mean() >= 0.98
    assert a.sum() == pytest.approx(b.sum(), rel=5e-3)
    assert r.stats.paths == int(z["paths"])
