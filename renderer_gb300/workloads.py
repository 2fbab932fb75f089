"""Deterministic synthetic workloads (seeded; no external data).

cornell_box()      256x256, 4x4 jittered spp, max depth 8, Russian roulette
                   from depth 3: five diffuse quads (2x2x2 room, white 0.73,
                   red and green side walls), a 0.5x0.5 ceiling area light of
                   radiance 15, a mirror and a glass (IOR 1.5) sphere, r=0.35,
                   pinhole camera with a 40 degree vertical field of view.
icosphere_scene()  an icosahedron subdivided 8 times (1,310,720 triangles)
                   displaced radially by 4-octave value noise of amplitude 0.1
                   (Phong kd 0.5, ks 0.3, exponent 50), a diffuse ground plane
                   of albedo 0.6, a 1024x512 lat-long sky (seeded gradient and a
                   0.5 degree sun disc of radiance 5e4) and one area light;
                   1024x1024, 8x8 spp, max depth 12.
two_rooms()        two diffuse rooms (each 4 x 3 x 3, albedo 0.7) sharing a
                   wall with a 0.2-wide door gap, a 0.3 x 0.3 area light of
                   radiance 200 on the far room's ceiling, the camera in the
                   near room, a glossy Blinn floor (exponent 200) and a
                   500,000-triangle displaced grid (500 x 500 quads) on the
                   near room's side wall; 1024x768. Lit almost only through
                   the door: the case path guiding is for (physical
                   semantics).
Spectra are BGR. Values given in RGB below are swapped on the way in.
"""
import numpy as np

from . import _abi
from .scene import SceneData, render_params

FOV_40 = 0.6981317  # 40 degrees in radians (the renderer's camera takes radians)


def bgr(rgb):
    return (float(rgb[2]), float(rgb[1]), float(rgb[0]))


# ---------------------------------------------------------------- Cornell box
def cornell_box(width=256, height=256):
    s = SceneData()
    white = s.add_material(_abi.MAT_DIFFUSE, kd=bgr((0.73, 0.73, 0.73)))
    red = s.add_material(_abi.MAT_DIFFUSE, kd=bgr((0.63, 0.065, 0.05)))
    green = s.add_material(_abi.MAT_DIFFUSE, kd=bgr((0.14, 0.45, 0.09)))
    mirror = s.add_material(_abi.MAT_MIRROR, coefficient=1.0)
    glass = s.add_material(_abi.MAT_TRANSPARENT, ior=1.5)
    s.quads = [
        ((-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1), white),      # floor
        ((-1, 2, -1), (-1, 2, 1), (1, 2, 1), (1, 2, -1), white),      # ceiling
        ((-1, 0, -1), (-1, 2, -1), (1, 2, -1), (1, 0, -1), white),    # back
        ((-1, 0, -1), (-1, 0, 1), (-1, 2, 1), (-1, 2, -1), red),      # left
        ((1, 0, -1), (1, 2, -1), (1, 2, 1), (1, 0, 1), green),        # right
    ]
    s.spheres = [((-0.45, 0.35, -0.3), 0.35, mirror), ((0.45, 0.35, 0.25), 0.35, glass)]
    # u x v = (0, -0.25, 0): the light faces down.
    s.lights = [dict(type=_abi.LIGHT_AREA, origin=(-0.25, 1.98, -0.25), u=(0.5, 0, 0), v=(0, 0, 0.5),
                     intensity=(15.0, 15.0, 15.0))]
    s.camera = dict(eye=(0, 1, 3.4), look_at=(0, 1, 0), up=(0, 1, 0), fov=FOV_40, width=width, height=height)
    return s


def cornell_params(max_depth=8, seed=0, x_samples=4, y_samples=4):
    return render_params(x_samples, y_samples, 0.5, max_depth, seed)


# ------------------------------------------------------------------ icosphere
_ICO_T = (1.0 + 5.0 ** 0.5) / 2.0
_ICO_V = np.array([(-1, _ICO_T, 0), (1, _ICO_T, 0), (-1, -_ICO_T, 0), (1, -_ICO_T, 0),
                   (0, -1, _ICO_T), (0, 1, _ICO_T), (0, -1, -_ICO_T), (0, 1, -_ICO_T),
                   (_ICO_T, 0, -1), (_ICO_T, 0, 1), (-_ICO_T, 0, -1), (-_ICO_T, 0, 1)], np.float64)
_ICO_F = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
                   (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
                   (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)


def icosphere(levels):
    """Unit icosphere: 20 * 4^levels triangles, 10 * 4^levels + 2 vertices."""
    V = _ICO_V / np.linalg.norm(_ICO_V, axis=1, keepdims=True)
    F = _ICO_F.copy()
    for _ in range(levels):
        nv = len(V)
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = V[a] + V[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = nv + inv.reshape(-1)
        nf = len(F)
        m01, m12, m20 = m[:nf], m[nf:2 * nf], m[2 * nf:]
        F = np.concatenate([np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
                            np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
        V = np.concatenate([V, mid])
    return V, F


def _splitmix64(z):
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _lattice(seed, i, j, k):
    h = (np.uint64(seed) ^ (i.astype(np.uint64) * np.uint64(0x8CB92BA72F3D8DD7))
         ^ (j.astype(np.uint64) * np.uint64(0xABC98388FB8FAC03))
         ^ (k.astype(np.uint64) * np.uint64(0xD6E8FEB86659FD93)))
    h = _splitmix64(h)
    return (h >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def value_noise(p, seed):
    """Trilinear value noise with smoothstep weights; lattice values in [-1, 1]
    from SplitMix64 of the integer coordinates."""
    f = np.floor(p)
    t = p - f
    w = t * t * (3.0 - 2.0 * t)
    i = f.astype(np.int64)
    out = np.zeros(len(p))
    # The lattice values over the box of cells the points touch, when that box
    # is small, hashed once and gathered (same values as hashing per point).
    lo = i.min(0) if len(p) else np.zeros(3, np.int64)
    ext = (i.max(0) + 2 - lo) if len(p) else np.ones(3, np.int64)
    table = None
    if int(np.prod(ext)) <= max(4 * len(p), 1 << 16):
        g = np.meshgrid(*[np.arange(lo[a], lo[a] + ext[a]) for a in range(3)], indexing="ij")
        table = _lattice(seed, g[0].ravel(), g[1].ravel(), g[2].ravel())
        rel = i - lo
        base = (rel[:, 0] * ext[1] + rel[:, 1]) * ext[2] + rel[:, 2]
    for dx in (0, 1):
        wx = w[:, 0] if dx else 1.0 - w[:, 0]
        for dy in (0, 1):
            wy = w[:, 1] if dy else 1.0 - w[:, 1]
            for dz in (0, 1):
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                if table is not None:
                    v = table[base + (dx * ext[1] + dy) * ext[2] + dz]
                else:
                    v = _lattice(seed, i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz)
                out += wx * wy * wz * v
    return out


def fbm(p, seed, octaves=4, base_freq=2.0, lacunarity=2.0, gain=0.5):
    """Fractal sum of value noise, normalised by the amplitude sum to [-1, 1]."""
    total, amp, norm, freq = np.zeros(len(p)), 1.0, 0.0, base_freq
    with np.errstate(over="ignore"):
        for o in range(octaves):
            total += amp * value_noise(p * freq, seed + 0x1000193 * o)
            norm += amp
            amp *= gain
            freq *= lacunarity
    return total / norm


def displaced_icosphere(levels=8, seed=0, amplitude=0.1, smooth_normals=True):
    """(tri_pos (N,9) float32, tri_nrm (N,9) float32 or None)."""
    V, F = icosphere(levels)
    r = 1.0 + amplitude * fbm(V, seed)
    P = V * r[:, None]
    tri = P[F]                                     # (N, 3, 3)
    pos = tri.reshape(-1, 9).astype(np.float32)
    if not smooth_normals:
        return pos, None
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])   # area-weighted
    N = np.zeros_like(P)
    for c in range(3):
        for k in range(3):
            N[:, c] += np.bincount(F[:, k], weights=fn[:, c], minlength=len(P))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    nrm = N[F].reshape(-1, 9).astype(np.float32)
    return pos, nrm


def latlong_dir(H, W):
    """Unit direction of each texel centre of a lat-long map: u = atan2(x, -z)
    / 2pi + 1/2 across, v = acos(y) / pi down (the library's lat-long lookup)."""
    v = (np.arange(H) + 0.5) / H
    u = (np.arange(W) + 0.5) / W
    theta = v[:, None] * np.pi
    phi = (u[None, :] - 0.5) * 2.0 * np.pi
    st = np.sin(theta)
    return np.stack([st * np.sin(phi), np.cos(theta) * np.ones_like(phi), -st * np.cos(phi)], -1)


def synthetic_sky(width=1024, height=512, seed=0, sun_radiance=5e4, sun_diameter_deg=0.5):
    """Lat-long HDR sky (H, W, 3) float32 BGR: zenith-to-horizon gradient, a
    darker ground, and a sun disc."""
    rng = np.random.default_rng(seed)
    d = latlong_dir(height, width)
    zen = np.array([0.25, 0.45, 1.0]) * rng.uniform(0.8, 1.2)
    hor = np.array([0.9, 0.9, 1.0]) * rng.uniform(0.8, 1.2)
    gnd = np.array([0.2, 0.18, 0.15])
    y = d[..., 1:2]
    sky = np.where(y >= 0, hor + (zen - hor) * np.sqrt(np.clip(y, 0, 1)), gnd)
    el = np.deg2rad(rng.uniform(25, 50))
    az = rng.uniform(0, 2 * np.pi)
    sun = np.array([np.cos(el) * np.sin(az), np.sin(el), -np.cos(el) * np.cos(az)])
    cosang = d @ sun
    disc = cosang >= np.cos(np.deg2rad(sun_diameter_deg / 2))
    # The texel containing the sun centre always carries it.
    row = min(int(np.arccos(sun[1]) / np.pi * height), height - 1)
    col = min(int((np.arctan2(sun[0], -sun[2]) / (2 * np.pi) + 0.5) * width), width - 1)
    disc[row, col] = True
    sky = np.where(disc[..., None], np.array([1.0, 0.95, 0.9]) * sun_radiance, sky)
    return sky[..., ::-1].astype(np.float32).copy(), sun   # RGB -> BGR


def icosphere_scene(levels=8, seed=0, width=1024, height=1024, env_size=(1024, 512), smooth_normals=True):
    s = SceneData()
    phong = s.add_material(_abi.MAT_PHONG, kd=bgr((0.5, 0.5, 0.5)), ks=bgr((0.3, 0.3, 0.3)), exponent=50.0)
    ground = s.add_material(_abi.MAT_DIFFUSE, kd=bgr((0.6, 0.6, 0.6)))
    pos, nrm = displaced_icosphere(levels, seed, 0.1, smooth_normals)
    s.tri_pos = pos
    s.tri_nrm = nrm
    s.tri_mat = np.full(len(pos), phong, np.int32)
    s.planes = [((0.0, 1.0, 0.0, 1.1), ground)]      # the plane y = -1.1
    sky, _ = synthetic_sky(env_size[0], env_size[1], seed)
    s.env = sky
    s.env_mapping = _abi.ENV_LATLONG
    s.lights = [dict(type=_abi.LIGHT_AREA, origin=(-0.5, 2.5, -0.5), u=(1, 0, 0), v=(0, 0, 1),
                     intensity=(10.0, 10.0, 10.0)),
                dict(type=_abi.LIGHT_ENV, intensity=(1.0, 1.0, 1.0))]
    s.camera = dict(eye=(0, 0.4, 3.2), look_at=(0, -0.1, 0), up=(0, 1, 0), fov=FOV_40, width=width,
                    height=height)
    return s


def icosphere_params(seed=0):
    return render_params(8, 8, 0.5, 12, seed)


# ------------------------------------------------------------------ two rooms
def displaced_grid(n, x0, x1, y0, y1, z_wall, depth, seed=0):
    """n x n quads (2 n^2 triangles) of the heightfield z = z_wall - depth *
    (1 + fbm(x, y)) / 2 over [x0, x1] x [y0, y1], with smooth normals."""
    xs = np.linspace(x0, x1, n + 1)
    ys = np.linspace(y0, y1, n + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    P2 = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1)
    h = 0.5 * (1.0 + fbm(P2 * 1.5, seed))
    P = np.stack([X.ravel(), Y.ravel(), z_wall - depth * h], 1)
    idx = np.arange((n + 1) * (n + 1)).reshape(n + 1, n + 1)
    a, b, c, d = idx[:-1, :-1].ravel(), idx[1:, :-1].ravel(), idx[1:, 1:].ravel(), idx[:-1, 1:].ravel()
    F = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)])
    tri = P[F]
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    N = np.zeros_like(P)
    for col in range(3):
        for k in range(3):
            N[:, col] += np.bincount(F[:, k], weights=fn[:, col], minlength=len(P))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    return tri.reshape(-1, 9).astype(np.float32), N[F].reshape(-1, 9).astype(np.float32)


def two_rooms(width=1024, height=768, mesh_quads=500, seed=0):
    s = SceneData()
    white = s.add_material(_abi.MAT_DIFFUSE, kd=bgr((0.7, 0.7, 0.7)))
    floor = s.add_material(_abi.MAT_BLINN, kd=bgr((0.25, 0.25, 0.25)), ks=bgr((0.45, 0.45, 0.45)), exponent=200.0)
    relief = s.add_material(_abi.MAT_DIFFUSE, kd=bgr((0.7, 0.6, 0.5)))
    q = []
    for x0 in (0.0, 4.0):   # per room: floor, ceiling
        q.append(((x0, 0, 0), (x0 + 4, 0, 0), (x0 + 4, 0, 3), (x0, 0, 3), floor))
        q.append(((x0, 3, 0), (x0, 3, 3), (x0 + 4, 3, 3), (x0 + 4, 3, 0), white))
    q.append(((0, 0, 0), (0, 0, 3), (0, 3, 3), (0, 3, 0), white))          # end wall x = 0
    q.append(((8, 0, 0), (8, 3, 0), (8, 3, 3), (8, 0, 3), white))          # end wall x = 8
    q.append(((0, 0, 0), (0, 3, 0), (8, 3, 0), (8, 0, 0), white))          # side wall z = 0
    q.append(((0, 0, 3), (8, 0, 3), (8, 3, 3), (0, 3, 3), white))          # side wall z = 3
    # shared wall x = 4 with a door gap z in [1.4, 1.6], y in [0, 2.2]
    q.append(((4, 0, 0), (4, 0, 1.4), (4, 3, 1.4), (4, 3, 0), white))
    q.append(((4, 0, 1.6), (4, 0, 3), (4, 3, 3), (4, 3, 1.6), white))
    q.append(((4, 2.2, 1.4), (4, 2.2, 1.6), (4, 3, 1.6), (4, 3, 1.4), white))
    s.quads = q
    pos, nrm = displaced_grid(mesh_quads, 0.6, 3.4, 0.2, 2.6, 2.97, 0.3, seed)
    s.tri_pos = pos
    s.tri_nrm = nrm
    s.tri_mat = np.full(len(pos), relief, np.int32)
    s.lights = [dict(type=_abi.LIGHT_AREA, origin=(5.85, 2.999, 1.35), u=(0.3, 0, 0), v=(0, 0, 0.3),
                     intensity=(200.0, 200.0, 200.0))]
    s.camera = dict(eye=(0.4, 1.5, 0.6), look_at=(4.0, 1.1, 1.8), up=(0, 1, 0), fov=1.0471976, width=width,
                    height=height)
    return s


def two_rooms_params(x_samples=1, y_samples=1, seed=0, max_depth=12, termination_prob=0.5):
    return render_params(x_samples, y_samples, termination_prob, max_depth, seed, semantics=_abi.SEM_PHYSICAL)


# ------------------------------------------------------------- batch of scenes
BATCH_RESOLUTIONS = (128, 256, 512, 1024)
# x_samples x y_samples pairs covering 4 to 256 samples per pixel
BATCH_SPP = ((2, 2), (2, 4), (4, 4), (4, 8), (8, 8), (8, 16), (16, 16))


def _rotation(rng):
    """A uniformly random rotation (QR of a Gaussian matrix, signs fixed)."""
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def _batch_material(s, rng):
    kind = int(rng.integers(4))
    if kind == 0:
        return s.add_material(_abi.MAT_DIFFUSE, kd=tuple(rng.uniform(0.2, 0.85, 3)))
    if kind == 1:
        return s.add_material(_abi.MAT_MIRROR, coefficient=1.0)
    if kind == 2:
        return s.add_material(_abi.MAT_TRANSPARENT, ior=1.5)
    kd = rng.uniform(0.1, 0.5, 3)
    return s.add_material(_abi.MAT_BLINN, kd=tuple(kd), ks=tuple(np.full(3, 0.9 - kd.max())),
                          exponent=float(rng.uniform(10.0, 500.0)))


def batch_scene(index, seed=0):
    """Scene `index` of the seeded batch: inside a diffuse 4 x 3 x 4 box open
    towards the camera, 1-3 noise-displaced meshes (heightfield patches,
    randomly rotated) with a log-uniform 10,000 to 2,000,000 triangles in
    total, 2-8 spheres, every object's material drawn uniformly from diffuse,
    mirror, glass (IOR 1.5) and Blinn (exponent 10-500), 1-4 ceiling area
    lights of radiance 5-50, a square resolution from 128 to 1024 and 4 to 256
    jittered samples per pixel. Returns (SceneData, gbrt_render_params): max
    depth 8, Russian roulette p = 0.5, reference semantics, BVH built on the
    GPU."""
    rng = np.random.default_rng([int(seed), int(index), 0xC3])
    s = SceneData()
    s.flags = _abi.SCENE_GPU_BUILD
    wall = s.add_material(_abi.MAT_DIFFUSE, kd=tuple(rng.uniform(0.5, 0.8, 3)))
    s.quads = [
        ((-2, 0, -2), (2, 0, -2), (2, 0, 2), (-2, 0, 2), wall),      # floor
        ((-2, 3, -2), (-2, 3, 2), (2, 3, 2), (2, 3, -2), wall),      # ceiling
        ((-2, 0, -2), (-2, 3, -2), (2, 3, -2), (2, 0, -2), wall),    # back
        ((-2, 0, -2), (-2, 0, 2), (-2, 3, 2), (-2, 3, -2), wall),    # left
        ((2, 0, -2), (2, 3, -2), (2, 3, 2), (2, 0, 2), wall),        # right
    ]
    n_tri = int(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
    k = int(rng.integers(1, 4))
    pos, nrm, mats = [], [], []
    for m in range(k):
        n = max(2, int(round(np.sqrt(n_tri / k / 2))))
        half = float(rng.uniform(0.4, 1.2))
        p, nn = displaced_grid(n, -half, half, -half, half, 0.0, 0.15 * half, seed=int(rng.integers(1 << 30)))
        R = _rotation(rng)
        c = np.array([rng.uniform(-1.0, 1.0), rng.uniform(0.8, 2.0), rng.uniform(-1.0, 1.0)])
        pos.append((p.reshape(-1, 3) @ R.T + c).reshape(-1, 9))
        nrm.append((nn.reshape(-1, 3) @ R.T).reshape(-1, 9))
        mats.append(np.full(len(p), _batch_material(s, rng), np.int32))
    s.tri_pos = np.concatenate(pos).astype(np.float32)
    s.tri_nrm = np.concatenate(nrm).astype(np.float32)
    s.tri_mat = np.concatenate(mats)
    for _ in range(int(rng.integers(2, 9))):
        r = float(rng.uniform(0.1, 0.45))
        c = (rng.uniform(-1.5, 1.5), rng.uniform(r, 2.5), rng.uniform(-1.5, 1.5))
        s.spheres.append((c, r, _batch_material(s, rng)))
    for _ in range(int(rng.integers(1, 5))):
        a, b = rng.uniform(0.3, 0.8, 2)
        x, z = rng.uniform(-1.9, 1.9 - a), rng.uniform(-1.9, 1.9 - b)
        le = float(rng.uniform(5.0, 50.0))
        # u x v points down (-y)
        s.lights.append(dict(type=_abi.LIGHT_AREA, origin=(x, 2.99, z), u=(a, 0, 0), v=(0, 0, b),
                             intensity=(le, le, le)))
    res = int(BATCH_RESOLUTIONS[rng.integers(len(BATCH_RESOLUTIONS))])
    xs, ys = BATCH_SPP[rng.integers(len(BATCH_SPP))]
    eye = (rng.uniform(-0.5, 0.5), rng.uniform(1.2, 1.8), rng.uniform(6.0, 7.0))
    s.camera = dict(eye=eye, look_at=(0, 1.5, 0), up=(0, 1, 0), fov=FOV_40, width=res, height=res)
    return s, render_params(xs, ys, 0.5, 8, seed=int(index))


def batch_scenes(n=64, seed=0):
    """The first n scenes of batch_scene's seeded sequence."""
    return [batch_scene(i, seed) for i in range(n)]


# ------------------------------------------------------ instanced terrain
def terrain(nx, nz, size_x, size_z, height, seed=0):
    """A heightfield of nx x nz quads (2 nx nz triangles) over [-size_x/2,
    size_x/2] x [-size_z/2, size_z/2], y = height (1 + fbm) / 2 from 4-octave
    value noise, with smooth (area-weighted) normals."""
    xs = np.linspace(-size_x / 2, size_x / 2, nx + 1)
    zs = np.linspace(-size_z / 2, size_z / 2, nz + 1)
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    P2 = np.stack([X.ravel() * 0.6, Z.ravel() * 0.6, np.zeros(X.size)], 1)
    Y = 0.5 * height * (1.0 + fbm(P2, seed))
    P = np.stack([X.ravel(), Y, Z.ravel()], 1)
    idx = np.arange((nx + 1) * (nz + 1)).reshape(nx + 1, nz + 1)
    a, b, c, d = idx[:-1, :-1].ravel(), idx[1:, :-1].ravel(), idx[1:, 1:].ravel(), idx[:-1, 1:].ravel()
    F = np.concatenate([np.stack([a, c, b], 1), np.stack([a, d, c], 1)])
    tri = P[F]
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    N = np.zeros_like(P)
    for col in range(3):
        for k in range(3):
            N[:, col] += np.bincount(F[:, k], weights=fn[:, col], minlength=len(P))
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    return tri.reshape(-1, 9).astype(np.float32), N[F].reshape(-1, 9).astype(np.float32)


def terrain_instances(seed=0, nx=2000, nz=1000, n_instances=8, n_spheres=200, width=3840, height=2160,
                      env_size=(2048, 1024), views=16):
    """Eight seeded copies (rotation about the vertical, scale 0.8-1.2,
    translation) of one 4,000,000-triangle noise-displaced terrain (2000 x
    1000 quads over 8 x 4 units) as instances of one mesh, 200 spheres of
    mixed materials (diffuse, mirror, glass 1.5, Blinn 10-500) above it, and
    a 2048 x 1024 lat-long sky with a sun as the only light. Returns
    (SceneData, cameras): `views` seeded camera poses at width x height."""
    rng = np.random.default_rng([int(seed), 0xC5])
    s = SceneData()
    s.env_mapping = _abi.ENV_LATLONG
    sky, _ = synthetic_sky(env_size[0], env_size[1], seed=int(seed), sun_radiance=2e4)
    s.env = sky
    s.lights = [dict(type=_abi.LIGHT_ENV, intensity=(1.0, 1.0, 1.0))]
    ground = s.add_material(_abi.MAT_DIFFUSE, kd=bgr((0.45, 0.4, 0.33)))
    pos, nrm = terrain(nx, nz, 8.0, 4.0, 0.8, int(seed))
    mi = s.add_mesh(pos, nrm, np.full(len(pos), ground, np.int32))
    for k in range(n_instances):
        ang = rng.uniform(0, 2 * np.pi)
        sc = rng.uniform(0.8, 1.2)
        c, sn = np.cos(ang), np.sin(ang)
        R = np.array([[c, 0, sn], [0, 1, 0], [-sn, 0, c]]) * sc
        t = ((k % 4) * 8.5 - 12.75 + rng.uniform(-0.5, 0.5), rng.uniform(-0.2, 0.2),
             (k // 4) * 8.5 - 4.25 + rng.uniform(-0.5, 0.5))
        M = np.zeros((3, 4))
        M[:, :3] = R
        M[:, 3] = t
        s.add_instance(M, mi)
    for _ in range(n_spheres):
        kind = int(rng.integers(4))
        if kind == 0:
            m = s.add_material(_abi.MAT_DIFFUSE, kd=tuple(rng.uniform(0.2, 0.85, 3)))
        elif kind == 1:
            m = s.add_material(_abi.MAT_MIRROR)
        elif kind == 2:
            m = s.add_material(_abi.MAT_TRANSPARENT, ior=1.5)
        else:
            kd = rng.uniform(0.1, 0.5, 3)
            m = s.add_material(_abi.MAT_BLINN, kd=tuple(kd), ks=tuple(np.full(3, 0.9 - kd.max())),
                               exponent=float(rng.uniform(10, 500)))
        r = float(rng.uniform(0.1, 0.6))
        s.spheres.append(((rng.uniform(-17, 17), rng.uniform(1.0, 3.5), rng.uniform(-8, 8)), r, m))
    cams = []
    for _ in range(views):
        a = rng.uniform(0, 2 * np.pi)
        d = rng.uniform(14, 24)
        eye = (d * np.cos(a), rng.uniform(3, 9), d * np.sin(a) * 0.7)
        look = (rng.uniform(-4, 4), rng.uniform(0, 1.5), rng.uniform(-2, 2))
        cams.append(dict(eye=eye, look_at=look, up=(0, 1, 0), fov=0.8, width=width, height=height))
    s.camera = cams[0]
    return s, cams
