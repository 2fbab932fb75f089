"""Thin Python handles over the C ABI, named after the renderer's interfaces.

  Context                     one CUDA device + stream (gbrt_ctx)
  GpuScene                    a scene in HBM with its BVH; intersect() is the
                              batched Intersectable::intersect (src/intersectable.h:40)
  UniDiPathTracingIntegrator  the integrator's option (src/unidipathtracingintegrator.cpp:34-46)
  PerPixelRenderer            render() of the image loop (src/perpixelrenderer.cpp:43-114)
"""
import ctypes as C
import weakref

import numpy as np

from . import _abi, check, lib
from .scene import SceneData, render_params

RAY_DTYPE = np.dtype([("org", np.float32, 3), ("tmin", np.float32), ("dir", np.float32, 3),
                      ("tmax", np.float32)])
HIT_DTYPE = np.dtype([("t", np.float32), ("prim", np.int32), ("u", np.float32), ("v", np.float32)])


def make_rays(org, dirs, tmin=0.001, tmax=np.inf):
    """Packs origins/directions (N, 3) into gbrt_ray records."""
    org = np.asarray(org, np.float32).reshape(-1, 3)
    dirs = np.asarray(dirs, np.float32).reshape(-1, 3)
    r = np.zeros(len(dirs), RAY_DTYPE)
    r["org"] = org
    r["dir"] = dirs
    r["tmin"] = tmin
    r["tmax"] = tmax
    return r


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """A device context. Closing it first closes the scenes created on it (a
    scene must not outlive its context)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        self.handle = None
        self._scenes = weakref.WeakSet()
        check(lib().gbrt_ctx_create(int(device), C.byref(h)))
        self.handle = h

    def trim(self):
        """Returns the memory the context's pool keeps between calls to the
        driver (gbrt_ctx_trim); the bytes it still holds."""
        v = C.c_uint64()
        check(lib().gbrt_ctx_trim(self.handle, C.byref(v)), self.handle)
        return v.value

    def close(self):
        for sc in list(self._scenes):
            sc.close()
        if self.handle:
            lib().gbrt_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuScene:
    """A scene uploaded to the device (gbrt_scene_create)."""

    def __init__(self, ctx: Context, data: SceneData):
        self.ctx = ctx
        self.data = data
        self.handle = None
        desc, keep = data.to_desc()
        h = C.c_void_p()
        check(lib().gbrt_scene_create(ctx.handle, C.byref(desc), C.byref(h)), ctx.handle)
        self.handle = h
        ctx._scenes.add(self)

    def info(self):
        nn, nl = C.c_int64(), C.c_int64()
        md = C.c_int32()
        sah, ms = C.c_double(), C.c_double()
        check(lib().gbrt_scene_info(self.handle, C.byref(nn), C.byref(nl), C.byref(md), C.byref(sah),
                                    C.byref(ms)))
        return dict(nodes=nn.value, leaves=nl.value, max_depth=md.value, sah_cost=sah.value,
                    build_ms=ms.value)

    def intersect(self, rays):
        """Closest hit of each ray (host arrays): structured array of HIT_DTYPE."""
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        hits = np.zeros(len(rays), HIT_DTYPE)
        check(lib().gbrt_trace_closest(self.handle, _ptr(rays), len(rays), _ptr(hits)), self.ctx.handle)
        return hits

    def occluded(self, rays, ignore_prim=None):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        occ = np.zeros(len(rays), np.uint8)
        ign = None if ignore_prim is None else np.ascontiguousarray(ignore_prim, np.int32)
        check(lib().gbrt_trace_any(self.handle, _ptr(rays), None if ign is None else _ptr(ign), len(rays),
                                   _ptr(occ)), self.ctx.handle)
        return occ.astype(bool)

    def close(self):
        if self.handle:
            lib().gbrt_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class UniDiPathTracingIntegrator:
    """The unidirectional integrator; its only option is the Russian-roulette
    termination probability (--pt-termination-prob)."""

    def __init__(self, termination_prob=0.5):
        self.termination_prob = float(termination_prob)


class PerPixelRenderer:
    """GPU PerPixelRenderer: same option names and defaults as the renderer
    (pt-integrator, pt-termination-prob, pt-x-samples, pt-y-samples)."""

    name = "pathtracing"

    @staticmethod
    def options():
        return {"pt-integrator": "unidi", "pt-termination-prob": 0.5, "pt-x-samples": 4, "pt-y-samples": 4}

    def __init__(self, scene: GpuScene, camera=None, options=None, seed=0, max_depth=5, batch_paths=0):
        opts = self.options()
        opts.update(options or {})
        if opts["pt-integrator"] != "unidi":
            raise ValueError("only the unidirectional integrator is provided")
        self.scene = scene
        self.camera = camera if camera is not None else scene.data.camera_struct()
        self.integrator = UniDiPathTracingIntegrator(opts["pt-termination-prob"])
        self.params = render_params(opts["pt-x-samples"], opts["pt-y-samples"], self.integrator.termination_prob,
                                    max_depth, seed, batch_paths=batch_paths)
        self.stats = _abi.Stats()

    def render(self, want_moments=False, stop_flag=None):
        """Returns the film (H, W, 3) float32 BGR, plus per-pixel sums and sums
        of squares (float64) when want_moments."""
        H, W = self.camera.height, self.camera.width
        film = np.zeros((H, W, 3), np.float32)
        s = np.zeros((H, W, 3), np.float64) if want_moments else None
        q = np.zeros((H, W, 3), np.float64) if want_moments else None
        stop = None if stop_flag is None else C.cast(C.pointer(stop_flag), C.c_void_p)
        check(lib().gbrt_render(self.scene.handle, C.byref(self.camera), C.byref(self.params), _ptr(film),
                                None if s is None else _ptr(s), None if q is None else _ptr(q), stop,
                                C.byref(self.stats)), self.scene.ctx.handle)
        return (film, s, q) if want_moments else film
