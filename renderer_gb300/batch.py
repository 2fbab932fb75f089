"""Batches of renders over the C ABI (gbrt_render_batch, gbrt_batch_autotune,
gbrt_render_batch_fused, gbrt_batch_autotune_fused).

No counterpart in the renderer, which renders one image per process
(src/main.cpp:182-265: one scene, one film). Two schedulers:

* streams (render_batch): each job is the same wavefront render as
  PerPixelRenderer.render; the jobs run concurrently on several CUDA streams
  of the context, longest first onto the least-loaded stream, and the host
  waits once for all of them;
* single launch (render_batch_fused): the jobs' paths share every wavefront,
  so each extend / shade / shadow launch serves many scenes and images; one
  wavefront is a captured CUDA graph, replayed until all paths are done.
"""
import ctypes as C

import numpy as np

from . import _abi, check, lib
from .runtime import Context, GpuScene


class BatchJob:
    """One image of a batch: a scene on the batch's context, its camera and
    render parameters (gbrt_render_params)."""

    def __init__(self, scene: GpuScene, camera, params):
        self.scene = scene
        self.camera = camera
        self.params = params


def _jobs_array(jobs, films):
    arr = (_abi.BatchJob * len(jobs))()
    for i, j in enumerate(jobs):
        arr[i].scene = j.scene.handle
        arr[i].camera = j.camera
        arr[i].params = j.params
        arr[i].film = films[i].ctypes.data_as(C.c_void_p) if films is not None else None
    return arr


def render_batch(ctx: Context, jobs, streams=0, batch_paths=0):
    """Renders every job. streams / batch_paths 0 take the context's tuned
    values. Returns (films, per-job device milliseconds, gbrt_batch_stats);
    each film is (H, W, 3) float32 BGR."""
    films = [np.zeros((j.camera.height, j.camera.width, 3), np.float32) for j in jobs]
    arr = _jobs_array(jobs, films)
    ms = (C.c_double * max(1, len(jobs)))()
    st = _abi.BatchStats()
    check(lib().gbrt_render_batch(ctx.handle, arr, len(jobs), int(streams), int(batch_paths), ms, C.byref(st)),
          ctx.handle)
    return films, np.array(ms[:len(jobs)], np.float64), st


def autotune(ctx: Context, jobs):
    """Chooses streams and wavefront size on a one-sample-per-pixel sample of
    the jobs and keeps them on the context. Returns (streams, batch_paths)."""
    arr = _jobs_array(jobs, None)
    s = C.c_int32()
    b = C.c_int64()
    check(lib().gbrt_batch_autotune(ctx.handle, arr, len(jobs), C.byref(s), C.byref(b)), ctx.handle)
    return s.value, b.value


def render_batch_fused(ctx: Context, jobs, wavefront_paths=0, pipelines=0, trace_block=0, shade_block=0):
    """Renders every job in shared wavefronts (one CUDA graph per wavefront,
    `pipelines` of them in flight). Zeros take the context's tuned schedule.
    Returns (films, per-job milliseconds to the wavefront that finished it,
    gbrt_batch_stats)."""
    films = [np.zeros((j.camera.height, j.camera.width, 3), np.float32) for j in jobs]
    arr = _jobs_array(jobs, films)
    ms = (C.c_double * max(1, len(jobs)))()
    st = _abi.BatchStats()
    sc = _abi.BatchSchedule(int(wavefront_paths), int(pipelines), int(trace_block), int(shade_block), 0)
    check(lib().gbrt_render_batch_fused(ctx.handle, arr, len(jobs), C.byref(sc), ms, C.byref(st)), ctx.handle)
    return films, np.array(ms[:len(jobs)], np.float64), st


def autotune_fused(ctx: Context, jobs):
    """Chooses the single-launch batch's schedule (wavefront size, pipelines
    in flight, tile sizes) on all jobs at one sample per pixel and keeps it on
    the context. Returns a dict of the choice."""
    arr = _jobs_array(jobs, None)
    sc = _abi.BatchSchedule()
    check(lib().gbrt_batch_autotune_fused(ctx.handle, arr, len(jobs), C.byref(sc)), ctx.handle)
    return {"wavefront_paths": sc.wavefront_paths, "pipelines": sc.pipelines, "trace_block": sc.trace_block,
            "shade_block": sc.shade_block}
