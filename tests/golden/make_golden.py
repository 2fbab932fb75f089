"""Generates the golden fixtures of tests/test_golden.py (run from the
repository root: python tests/golden/make_golden.py).

* probe_rows.hdr / probe_rows.npz: eight run-length-encoded scanlines
  (rows 316-323, through the centre) of the renderer's shipped angular light
  probe environmentmaps/campus_probe.hdr, re-wrapped with their own Radiance
  header, and their texels decoded by decode_radiance() below, a numpy
  restatement of the Radiance RGBE format (new-style run-length scanlines,
  mantissa * 2^(exponent - 136), BGR order as cv::imread returns it);
  also the full probe's shape and per-channel sums.
* cornell_rays.npz: 4,096 seeded rays on the 64x64 Cornell box (camera rays
  with jitter, and random rays from inside the box) and the oracle's closest
  hits (the renderer's median-split BVH, BVHNode::intersect).
* cornell_render.npz: the oracle's 32x32 Cornell-box image (2x2 spp, depth 8,
  seed 7, reference semantics) drawn with the counter-based stream that the
  GPU path tracer uses (SplitMix64 over seed, sample id and dimension).
* cornell_physical_mlt.npz: the same box under the physically based
  estimator (2x2 spp, depth 8, seed 9), and the oracle's Metropolis image
  (64 chains, 8 mutations per pixel, bootstrap 500, seed 2) with its normaliser b and
  acceptance count.

The probe is read from the renderer's source tree; the other fixtures need
only the oracle (oracle/binding.py builds it).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
HERE = os.path.join(ROOT, "tests", "golden")
# The renderer's source tree (its shipped light probe is read from it); the
# GBRT_REFERENCE_DIR environment variable overrides where it is looked for.
REFERENCE_DIR = os.environ.get("GBRT_REFERENCE_DIR", "/root/reference")
PROBE = os.path.join(REFERENCE_DIR, "environmentmaps", "campus_probe.hdr")
PROBE_ROWS = (316, 324)


def parse_header(data):
    """(width, height, offset of the first scanline) of a Radiance file."""
    pos = 0
    lines = []
    while True:
        end = data.index(b"\n", pos)
        line = data[pos:end]
        pos = end + 1
        if line == b"" and lines:
            break
        lines.append(line)
    if not lines[0].startswith(b"#?"):
        raise ValueError("not a Radiance file")
    end = data.index(b"\n", pos)
    res = data[pos:end].split()
    pos = end + 1
    if res[0] != b"-Y" or res[2] != b"+X":
        raise ValueError("only -Y H +X W images")
    return int(res[3]), int(res[1]), pos


def decode_radiance(data):
    """Radiance RGBE image -> ((H, W, 3) float32 BGR, list of (start, end)
    byte ranges of the scanlines)."""
    W, H, pos = parse_header(data)
    rgbe = np.zeros((H, W, 4), np.uint8)
    ranges = []
    for y in range(H):
        start = pos
        if data[pos] == 2 and data[pos + 1] == 2 and (data[pos + 2] << 8 | data[pos + 3]) == W:
            pos += 4
            for c in range(4):
                x = 0
                while x < W:
                    n = data[pos]
                    pos += 1
                    if n > 128:
                        rgbe[y, x:x + n - 128, c] = data[pos]
                        pos += 1
                        x += n - 128
                    else:
                        rgbe[y, x:x + n, c] = np.frombuffer(data[pos:pos + n], np.uint8)
                        pos += n
                        x += n
        else:  # flat scanline
            rgbe[y] = np.frombuffer(data[pos:pos + 4 * W], np.uint8).reshape(W, 4)
            pos += 4 * W
        ranges.append((start, pos))
    e = rgbe[..., 3].astype(np.int32)
    f = np.where(e > 0, np.ldexp(1.0, e - 136), 0.0)
    rgb = rgbe[..., :3].astype(np.float64) * f[..., None]
    return rgb[..., ::-1].astype(np.float32), ranges


def make_probe():
    if not os.path.exists(PROBE):
        raise SystemExit("make_golden.py: the renderer's light probe %s is missing; point GBRT_REFERENCE_DIR at "
                         "the renderer's source tree" % PROBE)
    data = open(PROBE, "rb").read()
    img, ranges = decode_radiance(data)
    W = img.shape[1]
    r0, r1 = PROBE_ROWS
    body = data[ranges[r0][0]:ranges[r1 - 1][1]]
    header = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n" % (r1 - r0, W)
    with open(os.path.join(HERE, "probe_rows.hdr"), "wb") as f:
        f.write(header + body)
    rows, _ = decode_radiance(header + body)
    assert np.array_equal(rows, img[r0:r1])
    np.savez_compressed(os.path.join(HERE, "probe_rows.npz"), texels=rows, full_shape=np.array(img.shape),
                        full_sums=img.astype(np.float64).sum((0, 1)))


def make_cornell():
    from oracle.binding import OracleScene
    from renderer_gb300 import workloads
    from renderer_gb300.runtime import make_rays

    s = workloads.cornell_box(64, 64)
    o = OracleScene(s)
    rng = np.random.default_rng(20261203)
    cam = s.camera
    eye, at, up = (np.array(cam[k], np.float64) for k in ("eye", "look_at", "up"))
    w = eye - at
    w /= np.linalg.norm(w)
    u = np.cross(up, w)
    u /= np.linalg.norm(u)
    v = np.cross(w, u)
    t = np.tan(cam["fov"] / 2)
    px, py = rng.random(2048) * 64, rng.random(2048) * 64
    x = -t + 2 * t * (px + 0.5) / 64
    y = t - 2 * t * (py + 0.5) / 64
    d_cam = x[:, None] * u + y[:, None] * v - w
    org = rng.uniform([-0.9, 0.1, -0.9], [0.9, 1.9, 0.9], (2048, 3))
    d_rnd = rng.normal(size=(2048, 3))
    rays = make_rays(np.concatenate([np.broadcast_to(eye, d_cam.shape), org]), np.concatenate([d_cam, d_rnd]))
    hits = o.intersect(rays)
    np.savez_compressed(os.path.join(HERE, "cornell_rays.npz"), rays=rays, hits=hits)

    s = workloads.cornell_box(32, 32)
    params = workloads.cornell_params(max_depth=8, seed=7, x_samples=2, y_samples=2)
    out = OracleScene(s).render(s.camera_struct(), params, rng_mode=1)
    np.savez_compressed(os.path.join(HERE, "cornell_render.npz"), film=out["film"], paths=out["paths"],
                        rays=out["rays"], shadow_rays=out["shadow_rays"])

    # the physically based estimator on the same box, and the Metropolis
    # renderer (64 chains, 8 mutations per pixel, bootstrap 500)
    from renderer_gb300 import _abi
    from renderer_gb300.chains import mlt_params
    from renderer_gb300.scene import render_params
    phys = OracleScene(s).render(s.camera_struct(), render_params(2, 2, 0.5, 8, 9, semantics=_abi.SEM_PHYSICAL),
                                 rng_mode=1)
    mlt = OracleScene(s).render_mlt(s.camera_struct(), render_params(1, 1, 0.0, 5, 2), mlt_params(8, 500), chains=64)
    np.savez_compressed(os.path.join(HERE, "cornell_physical_mlt.npz"), phys_film=phys["film"],
                        mlt_film=mlt["film"], mlt_b=mlt["b"], mlt_accepted=mlt["accepted"],
                        mlt_mutations=mlt["mutations"])


if __name__ == "__main__":
    os.makedirs(HERE, exist_ok=True)
    make_probe()
    make_cornell()
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))
