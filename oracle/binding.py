"""ctypes binding of oracle/_build/liboracle.so (TEST INFRASTRUCTURE ONLY).

Builds the library on first use when it is missing (oracle/build.sh).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from renderer_gb300 import _abi
from renderer_gb300.runtime import HIT_DTYPE, RAY_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
# The same source built with the renderer's Release flags, for the timed CPU
# baseline only (its float results may differ from the parity build's in the
# last bits).
TIME_LIB_PATH = os.path.join(HERE, "_build", "liboracle_time.so")
_libs = {}


def build():
    subprocess.run(["sh", os.path.join(HERE, "build.sh")], check=True)
    return LIB_PATH


def lib(timing=False):
    """The parity build (default) or, with timing, the timing build."""
    path = TIME_LIB_PATH if timing else LIB_PATH
    if path not in _libs:
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.orc_scene_create.restype = P
        L.orc_scene_create.argtypes = [C.POINTER(_abi.SceneDesc), C.c_int]
        L.orc_scene_destroy.argtypes = [P]
        L.orc_scene_prims.restype = C.c_int
        L.orc_scene_prims.argtypes = [P]
        L.orc_trace_closest.argtypes = [P, P, C.c_int64, P, C.c_int]
        L.orc_trace_any.argtypes = [P, P, P, C.c_int64, P, C.c_int]
        L.orc_render.restype = C.c_int
        L.orc_render.argtypes = [P, C.POINTER(_abi.Camera), C.POINTER(_abi.RenderParams), C.c_int, C.c_int, C.c_int,
                                 C.c_int, P, P, P, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                 C.POINTER(C.c_uint64)]
        L.orc_camera_ray.argtypes = [C.POINTER(_abi.Camera), C.c_double, C.c_double, P]
        L.orc_tonemap.argtypes = [P, C.c_int, C.c_int, C.c_float, P]
        L.orc_render_mlt.restype = C.c_int
        L.orc_render_mlt.argtypes = [P, C.POINTER(_abi.Camera), C.POINTER(_abi.RenderParams),
                                     C.POINTER(_abi.MltParams), C.c_int64, P, C.POINTER(C.c_double),
                                     C.POINTER(C.c_uint64)]
        L.orc_render_erpt.restype = C.c_int
        L.orc_render_erpt.argtypes = [P, C.POINTER(_abi.Camera), C.POINTER(_abi.RenderParams),
                                      C.POINTER(_abi.ErptParams), P, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
        L.orc_stream_u.restype = C.c_float
        L.orc_stream_u.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32]
        _libs[path] = L
    return _libs[path]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleScene:
    """The renderer's scene (IntersectableList of lights + geometry, median-split
    BVH or a plain list) restated on the CPU."""

    def __init__(self, data, use_bvh=True, timing=False):
        """timing: on the timing build (the CPU baseline), not the parity build."""
        desc, keep = data.to_desc()
        self.data = data
        self._L = lib(timing)
        self.handle = self._L.orc_scene_create(C.byref(desc), 1 if use_bvh else 0)
        if not self.handle:
            raise RuntimeError("orc_scene_create failed")

    def intersect(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        hits = np.zeros(len(rays), HIT_DTYPE)
        self._L.orc_trace_closest(self.handle, _ptr(rays), len(rays), _ptr(hits), threads)
        return hits

    def occluded(self, rays, ignore_prim=None, threads=0):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        occ = np.zeros(len(rays), np.uint8)
        ign = None if ignore_prim is None else np.ascontiguousarray(ignore_prim, np.int32)
        self._L.orc_trace_any(self.handle, _ptr(rays), _ptr(ign), len(rays), _ptr(occ), threads)
        return occ.astype(bool)

    def render(self, camera, params, rng_mode=0, rows=None, threads=0, row_step=1):
        """Returns dict(film, sum, sumsq, paths, rays, shadow_rays) for rows
        r0, r0 + row_step, ... < r1 (all rows by default)."""
        H, W = camera.height, camera.width
        r0, r1 = rows if rows is not None else (0, H)
        film = np.zeros((H, W, 3), np.float32)
        s = np.zeros((H, W, 3), np.float64)
        q = np.zeros((H, W, 3), np.float64)
        paths, rays, sh = C.c_uint64(), C.c_uint64(), C.c_uint64()
        rc = self._L.orc_render(self.handle, C.byref(camera), C.byref(params), rng_mode, r0, r1, row_step, _ptr(film), _ptr(s),
                              _ptr(q), threads, C.byref(paths), C.byref(rays), C.byref(sh))
        if rc != 0:
            raise RuntimeError("orc_render failed")
        return dict(film=film, sum=s, sumsq=q, paths=paths.value, rays=rays.value, shadow_rays=sh.value)

    def render_mlt(self, camera, params, mp, chains):
        """MetropolisRenderer with `chains` chains. Returns dict(film, b,
        paths, mutations, accepted, chains)."""
        film = np.zeros((camera.height, camera.width, 3), np.float32)
        b = C.c_double()
        counts = (C.c_uint64 * 4)()
        if self._L.orc_render_mlt(self.handle, C.byref(camera), C.byref(params), C.byref(mp), int(chains), _ptr(film),
                                C.byref(b), counts) != 0:
            raise RuntimeError("orc_render_mlt failed")
        return dict(film=film, b=b.value, paths=counts[0], mutations=counts[1], accepted=counts[2], chains=counts[3])

    def render_erpt(self, camera, params, ep):
        """EnergyRedistributionRenderer. Returns dict(film, ed, paths,
        mutations, accepted, chains)."""
        film = np.zeros((camera.height, camera.width, 3), np.float32)
        ed = C.c_double()
        counts = (C.c_uint64 * 4)()
        if self._L.orc_render_erpt(self.handle, C.byref(camera), C.byref(params), C.byref(ep), _ptr(film), C.byref(ed),
                                 counts) != 0:
            raise RuntimeError("orc_render_erpt failed")
        return dict(film=film, ed=ed.value, paths=counts[0], mutations=counts[1], accepted=counts[2], chains=counts[3])

    def close(self):
        if self.handle:
            self._L.orc_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def camera_ray(camera, px, py):
    r = np.zeros(1, RAY_DTYPE)
    lib().orc_camera_ray(C.byref(camera), px, py, _ptr(r))
    return r[0]


def stream_u(seed, sample_id, dim):
    return lib().orc_stream_u(seed, sample_id, dim)


def tonemap(film, gamma=2.2):
    """Tonemapper::map of a (H, W, 3) BGR film -> (H, W, 3) RGB uint8."""
    film = np.ascontiguousarray(film, np.float32)
    out = np.zeros(film.shape, np.uint8)
    lib().orc_tonemap(_ptr(film), film.shape[1], film.shape[0], gamma, _ptr(out))
    return out
