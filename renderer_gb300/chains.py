"""The renderer's Markov-chain renderers over the C ABI (gbrt_render_mlt,
gbrt_render_erpt), with the renderer's option names.

MetropolisRenderer (src/metropolisrenderer.cpp:56-201, options at :203-212)
and EnergyRedistributionRenderer (src/energyredistributionrenderer.cpp:38-135,
options at :137-145): primary-sample-space chains whose proposals are traced
by the same wavefront kernels as the per-pixel renderer, every chain advanced
one mutation per wavefront.
"""
import ctypes as C

import numpy as np

from . import _abi, check, lib
from .runtime import GpuScene
from .scene import render_params


def mlt_params(mutations=16, bootstrap=10000, large_step_prob=0.1, termination_prob=0.5, chains=0):
    return _abi.MltParams(int(mutations), int(bootstrap), float(large_step_prob), float(termination_prob), int(chains))


def erpt_params(mutations=100, x_samples=2, y_samples=2, batch_chains=0):
    return _abi.ErptParams(int(mutations), int(x_samples), int(y_samples), 0, int(batch_chains))


class MetropolisRenderer:
    """GPU MetropolisRenderer ("metropolis"): met-large-step-prob,
    met-termination-prob, met-bootstrap, met-mutations, plus the number of
    parallel chains (the renderer runs one per OpenMP thread)."""

    name = "metropolis"

    @staticmethod
    def options():
        return {"met-large-step-prob": 0.1, "met-termination-prob": 0.5, "met-bootstrap": 10000,
                "met-mutations": 16}

    def __init__(self, scene: GpuScene, camera=None, options=None, seed=0, max_depth=5, chains=0):
        opts = self.options()
        opts.update(options or {})
        self.scene = scene
        self.camera = camera if camera is not None else scene.data.camera_struct()
        self.params = render_params(1, 1, 0.0, max_depth, seed)
        self.mp = mlt_params(opts["met-mutations"], opts["met-bootstrap"], opts["met-large-step-prob"],
                             opts["met-termination-prob"], chains)
        self.stats = _abi.ChainStats()

    def render(self):
        film = np.zeros((self.camera.height, self.camera.width, 3), np.float32)
        check(lib().gbrt_render_mlt(self.scene.handle, C.byref(self.camera), C.byref(self.params), C.byref(self.mp),
                                    film.ctypes.data_as(C.c_void_p), C.byref(self.stats)), self.scene.ctx.handle)
        return film


class EnergyRedistributionRenderer:
    """GPU EnergyRedistributionRenderer ("energyredist"): erpt-mutations,
    erpt-x-samples, erpt-y-samples."""

    name = "energyredist"

    @staticmethod
    def options():
        return {"erpt-mutations": 100, "erpt-x-samples": 2, "erpt-y-samples": 2}

    def __init__(self, scene: GpuScene, camera=None, options=None, seed=0, max_depth=5, batch_chains=0):
        opts = self.options()
        opts.update(options or {})
        self.scene = scene
        self.camera = camera if camera is not None else scene.data.camera_struct()
        self.params = render_params(1, 1, 0.0, max_depth, seed)
        self.ep = erpt_params(opts["erpt-mutations"], opts["erpt-x-samples"], opts["erpt-y-samples"], batch_chains)
        self.stats = _abi.ChainStats()

    def render(self):
        film = np.zeros((self.camera.height, self.camera.width, 3), np.float32)
        check(lib().gbrt_render_erpt(self.scene.handle, C.byref(self.camera), C.byref(self.params), C.byref(self.ep),
                                     film.ctypes.data_as(C.c_void_p), C.byref(self.stats)), self.scene.ctx.handle)
        return film
