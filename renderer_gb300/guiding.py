"""Neural path guiding over the C ABI (gbrt_guide_*, gbrt_render_guided).

No counterpart in the renderer: its integrators sample BSDFs only
(src/unidipathtracingintegrator.cpp:34-46). A Guide is a small MLP on the
device that maps (position, normal, outgoing direction) to a mixture of 8 von
Mises-Fisher lobes; render_guided samples non-specular vertices from it with
probability guide_fraction (one-sample MIS with the BSDF) under the physical
estimator and trains it online on the tracer's own radiance samples.
"""
import ctypes as C

import numpy as np

from . import _abi, check, lib
from .runtime import Context, GpuScene


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def scene_bounds(scene: GpuScene):
    b = (C.c_float * 6)()
    check(lib().gbrt_scene_bounds(scene.handle, b))
    return np.array(b, np.float32)


class Guide:
    """A guiding network on a context's device (gbrt_guide_create)."""

    def __init__(self, ctx: Context, bounds, seed=0):
        self.ctx = ctx
        self.handle = None
        self.bounds = np.ascontiguousarray(bounds, np.float32).reshape(6)
        h = C.c_void_p()
        check(lib().gbrt_guide_create(ctx.handle, self.bounds.ctypes.data_as(C.POINTER(C.c_float)),
                                      int(seed) & (2**64 - 1), C.byref(h)), ctx.handle)
        self.handle = h
        ctx._scenes.add(self)  # closed before its context

    def weights(self):
        w = np.zeros(_abi.GUIDE_PARAMS, np.float32)
        check(lib().gbrt_guide_get_weights(self.handle, _ptr(w), w.size), self.ctx.handle)
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32).reshape(-1)
        check(lib().gbrt_guide_set_weights(self.handle, _ptr(w), w.size), self.ctx.handle)

    def get_state(self):
        """Checkpoint of training: {"params", "adam_m", "adam_v" (GUIDE_PARAMS
        float32 each), "step"}."""
        n = _abi.GUIDE_PARAMS
        out = {k: np.zeros(n, np.float32) for k in ("params", "adam_m", "adam_v")}
        step = C.c_int64()
        check(lib().gbrt_guide_get_state(self.handle, _ptr(out["params"]), _ptr(out["adam_m"]),
                                         _ptr(out["adam_v"]), C.byref(step)), self.ctx.handle)
        out["step"] = step.value
        return out

    def set_state(self, state):
        """Resumes training from a get_state checkpoint."""
        a = [np.ascontiguousarray(state[k], np.float32).reshape(-1) for k in ("params", "adam_m", "adam_v")]
        check(lib().gbrt_guide_set_state(self.handle, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), int(state["step"])),
              self.ctx.handle)

    def eval(self, inputs):
        """inputs (N, 9): point, normal facing the viewer, outgoing direction.
        Returns (N, 40): lobe weights [8], then (mean xyz, kappa) per lobe."""
        x = np.ascontiguousarray(inputs, np.float32).reshape(-1, _abi.GUIDE_INPUT)
        out = np.zeros((len(x), _abi.GUIDE_OUTPUT), np.float32)
        check(lib().gbrt_guide_eval(self.handle, _ptr(x), len(x), _ptr(out)), self.ctx.handle)
        return out

    def gradient(self, samples):
        """samples (N, 13): point, normal, outgoing, sampled direction, weight.
        Returns (gradient of the loss, loss)."""
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, _abi.GUIDE_SAMPLE)
        g = np.zeros(_abi.GUIDE_PARAMS, np.float32)
        loss = C.c_float()
        check(lib().gbrt_guide_gradient(self.handle, _ptr(s), len(s), _ptr(g), C.byref(loss)), self.ctx.handle)
        return g, loss.value

    def train_step(self, samples, learning_rate=1e-2):
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, _abi.GUIDE_SAMPLE)
        loss = C.c_float()
        check(lib().gbrt_guide_train_step(self.handle, _ptr(s), len(s), float(learning_rate), C.byref(loss)),
              self.ctx.handle)
        return loss.value

    def close(self):
        if self.handle:
            lib().gbrt_guide_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def guide_params(guide_fraction=0.5, passes=0, train_passes=0, steps_per_pass=0, batch_samples=1 << 18,
                 learning_rate=1e-2, time_budget_ms=0.0, guide_depth=0, flags=0, warmup_steps=0,
                 late_pass_samples=0):
    p = _abi.GuideParams()
    p.guide_fraction = guide_fraction
    p.passes = passes
    p.train_passes = train_passes
    p.steps_per_pass = steps_per_pass
    p.batch_samples = batch_samples
    p.learning_rate = learning_rate
    p.time_budget_ms = time_budget_ms
    p.guide_depth = guide_depth
    p.flags = flags
    p.warmup_steps = warmup_steps
    p.late_pass_samples = late_pass_samples
    return p


def render_guided(scene: GpuScene, camera, params, guide=None, gp=None):
    """Film (H, W, 3) float32 BGR and the call's gbrt_guide_stats."""
    gp = gp if gp is not None else guide_params(passes=1)
    film = np.zeros((camera.height, camera.width, 3), np.float32)
    st = _abi.GuideStats()
    check(lib().gbrt_render_guided(scene.handle, C.byref(camera), C.byref(params),
                                   guide.handle if guide is not None else None, C.byref(gp), _ptr(film),
                                   C.byref(st)), scene.ctx.handle)
    return film, st
