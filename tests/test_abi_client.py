"""The C ABI from C++ alone: tests/abi_client.cpp includes only
include/gbrt.h and links libgbrt.so, as the renderer's own binding would
(parse a scene file, create the scene, gbrt_render with the renderer's
options, gbrt_render_mlt, gbrt_write_image). CPU: it compiles and links with
g++. GPU: it runs, and its film is the ctypes binding's film of the same
render (same seed: the same paths)."""
import os
import subprocess

import numpy as np
import pytest

from renderer_gb300 import LIB_PATH

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def client(gbrt_built, tmp_path_factory):
    d = tmp_path_factory.mktemp("client")
    exe = d / "abi_client"
    lib_dir = os.path.dirname(LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_client.cpp"), "-L", lib_dir, "-lgbrt",
                    "-Wl,-rpath," + lib_dir, "-o", str(exe)], check=True)
    return exe


def test_client_builds_against_the_header_alone(client):
    assert os.path.exists(client)
    r = subprocess.run([str(client)], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
def test_client_renders_the_bindings_image(client, tmp_path, ctx):
    from renderer_gb300 import GpuScene, PerPixelRenderer, workloads
    from renderer_gb300.scenefile import load_scene, read_hdr, write_scene
    s = workloads.cornell_box(64, 48)
    scene = write_scene(s, str(tmp_path / "cornell.scene"))
    out = tmp_path / "cornell.pfm"
    r = subprocess.run([str(client), scene, str(out), "2", "2", "6"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    tag, paths, mean, mmean = r.stdout.split()
    assert tag == "ok" and int(paths) == 64 * 48 * 4
    t = load_scene(scene)
    film = PerPixelRenderer(GpuScene(ctx, t), options={"pt-x-samples": 2, "pt-y-samples": 2}, seed=1,
                            max_depth=6).render()
    assert float(mean) == pytest.approx(float(film.mean()), rel=1e-5)
    assert float(mmean) == pytest.approx(float(film.mean()), rel=0.3)
    img = read_hdr(str(out))
    assert img.shape == film.shape and np.allclose(img, film, rtol=1e-5, atol=1e-6)
