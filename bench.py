"""Benchmark of the GB300 path-tracing hot path (one JSON line on stdout).

Workload (the headline configuration): the 1,310,720-triangle displaced
icosphere with a diffuse ground plane, a 1024x512 lat-long sky with a sun
disc and one area light; 1024x1024 pixels, 8x8 jittered samples per pixel
(67,108,864 camera samples per frame), maximum path length 12, Russian
roulette with termination probability 0.5, the renderer's estimator
("reference semantics"). Synthetic, seeded data; no files are read.

A step is one full frame. value = camera samples (paths) per second over the
K timed frames, inputs resident in HBM (gbrt_render_device); e2e = the same
metric through the C ABI with host buffers (gbrt_render: film copied back to
the host every frame). The roofline entry covers the dominant kernel, the
closest-hit traversal (k_extend), timed with CUDA events on its own stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the renderer's own
PerPixelRenderer path (the oracle, built from oracle/) on all host cores, on a
bounded sample of rows of the same workload per step. With torchrun (N > 1)
every rank renders its own frame (replicas; the path needs no exchange).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("icosphere-1.31M-tri, 1024x1024, 8x8 spp, max depth 12, RR p=0.5, lat-long sky 1024x512 "
            "+ sun + area light, reference semantics")


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return ws, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(x, dist):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def extend_traffic():
    """The committed ncu capture of every k_extend launch of one frame of
    this workload (profiles/k_extend_icosphere_traffic.json): DRAM and L2
    bytes per camera ray and per bounce ray, or None."""
    p = os.path.join(ROOT, "profiles", "k_extend_icosphere_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(scene, cam, params, rows, threads=0):
    """The oracle (CPU restatement of the renderer's PerPixelRenderer path,
    reference semantics, per-row generators) on a bounded, evenly spread
    sample of rows. Returns (paths/s, paths, seconds, threads)."""
    from oracle.binding import OracleScene
    H = cam.height
    step = max(1, H // rows)
    o = scene if hasattr(scene, "render") else OracleScene(scene, timing=True)
    t = time.perf_counter()
    r = o.render(cam, params, rng_mode=0, rows=(step // 2, H), row_step=step, threads=threads)
    dt = time.perf_counter() - t
    return r["paths"] / dt, r["paths"], dt, (threads or os.cpu_count())


def run_reference(args, ws, rank, dist):
    if rank != 0:
        return
    from oracle.binding import OracleScene
    from renderer_gb300 import workloads
    s = workloads.icosphere_scene(levels=8)
    cam = s.camera_struct()
    params = workloads.icosphere_params()
    t = time.perf_counter()
    o = OracleScene(s, timing=True)
    build_s = time.perf_counter() - t
    rows = args.reference_rows
    for _ in range(args.warmup):
        cpu_baseline(o, cam, params, rows)
    rates, paths, secs = [], 0, 0.0
    for _ in range(args.steps):
        rate, n, dt, cores = cpu_baseline(o, cam, params, rows)
        rates.append(rate)
        paths += n
        secs += dt
    value = paths / secs
    sample = "%d evenly spaced rows of 1024 (x 1024 px x 64 spp = %d paths) per step" % (rows, paths // args.steps)
    line = {"impl": "reference", "metric": "paths/s", "value": value, "unit": "paths/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": {"workload": WORKLOAD, "scene_build_s": build_s},
            "cpu_baseline": {"value": value, "unit": "paths/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


SPP_DEFAULT = [16, 32, 64, 128, 256, 512]
GUIDED_WORKLOAD = ("two rooms 4x3x3 (albedo 0.7) joined by a 0.2-wide door, 0.3x0.3 area light of radiance 200 "
                   "in the far room, 500,000-triangle displaced grid, Blinn floor (exponent 200), 1024x768, "
                   "physical semantics, max depth 12, RR p=0.5")


def interp_time(curve, target):
    """Time at which relMSE reaches target, log-log interpolation along a
    (ms, relmse) curve sorted by time; None when the curve never gets there."""
    import math
    pts = sorted(curve)
    for (t0, e0), (t1, e1) in zip(pts, pts[1:]):
        if e0 > target >= e1:
            f = (math.log(target) - math.log(e0)) / (math.log(e1) - math.log(e0))
            return math.exp(math.log(t0) + f * (math.log(t1) - math.log(t0)))
    if pts and pts[0][1] <= target:
        return pts[0][0]
    return None


def run_guided(args):
    """Equal-time relMSE of guided against plain GPU path tracing on the
    two-room scene, both against a high-sample render of the plain physical
    estimator accumulated in FP64; plus the network kernels' tensor rates."""
    import numpy as np

    from renderer_gb300 import _abi, workloads
    from renderer_gb300.guiding import Guide, guide_params, render_guided, scene_bounds
    from renderer_gb300.runtime import Context, GpuScene

    from renderer_gb300.scene import render_params

    ctx = Context(0)
    terrain = args.guided_scene == "terrain"
    if terrain:
        s, cams = workloads.terrain_instances(seed=0, nx=args.terrain_nx, nz=args.terrain_nx // 2)
        full_cam = dict(cams[0])
        s.camera = dict(cams[0], width=args.guided_width, height=args.guided_height)
        workload = ("instanced terrain (8 x 4M-triangle instances, 200 spheres, sky), view 0 at %dx%d, physical "
                    "semantics, max depth 16, RR p=0.5" % (args.guided_width, args.guided_height))
    else:
        s = workloads.two_rooms(1024, 768, mesh_quads=500)
        workload = GUIDED_WORKLOAD
    gs = GpuScene(ctx, s)
    cam = s.camera_struct()
    bounds = scene_bounds(gs)

    def prm(xs, seed, flags=0):
        if terrain:
            return render_params(xs, xs, 0.5, 16, seed, semantics=_abi.SEM_PHYSICAL, flags=flags)
        p = workloads.two_rooms_params(xs, xs, seed=seed)
        p.flags = flags
        return p

    gflags = (0 if args.absolute_weights else _abi.GUIDE_PIXEL_RELATIVE) | (
        _abi.GUIDE_PRODUCT if args.product_target else 0) | (_abi.GUIDE_ASYNC_TRAINING if args.async_train else 0)

    def train_gp(budget_ms=0.0, passes=0):
        return guide_params(args.guide_fraction, passes=passes, train_passes=args.train_passes,
                            steps_per_pass=args.train_steps, batch_samples=1 << 18, learning_rate=1e-2,
                            time_budget_ms=budget_ms, guide_depth=args.guide_depth, flags=gflags,
                            warmup_steps=args.warmup_steps, late_pass_samples=args.late_pass_samples)

    if args.profile:
        g = Guide(ctx, bounds, seed=1)
        gp = guide_params(args.guide_fraction, passes=2, train_passes=2, steps_per_pass=2, batch_samples=1 << 18)
        _, st = render_guided(gs, cam, prm(1, 1), g, gp)
        _, st2 = render_guided(gs, cam, prm(1, 2), g, guide_params(args.guide_fraction, passes=1))
        print(json.dumps({"profile": "guided", "train_steps": st.train_steps, "infer_rows": st2.infer_rows}))
        return

    ref_spp = max(1, args.ref_spp // 64) * 64
    if args.ref_cache and os.path.exists(args.ref_cache):
        z = np.load(args.ref_cache)
        ref, ref_ms = z["film"], float(z["ms"])
        assert int(z["spp"]) == ref_spp, "cached reference has another sample count"
    elif args.ref_guided:
        # Both estimators are unbiased; a guided reference converges where the
        # plain one keeps rare, very bright samples (a sun seen through BSDF
        # sampling) at this sample count.
        g = Guide(ctx, bounds, seed=3)
        ref, st = render_guided(gs, cam, prm(8, 1), g, train_gp(passes=ref_spp // 64))
        ref_ms = st.total_ms
        g.close()
        if args.ref_cache:
            np.savez(args.ref_cache, film=ref, ms=ref_ms, spp=ref_spp)
    else:
        ref, st = render_guided(gs, cam, prm(8, 1), None, guide_params(passes=ref_spp // 64))
        ref_ms = st.total_ms
        if args.ref_cache:
            np.savez(args.ref_cache, film=ref, ms=ref_ms, spp=ref_spp)

    def relmse(x):
        return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))

    if args.headroom:
        # What a guide trained far beyond the equal-time budget gains at equal
        # samples per pixel: train untimed (8 Adam steps of 2^18 samples after
        # each training pass), then render with the weights frozen.
        n = args.headroom_spp
        img, st = render_guided(gs, cam, prm(1, 11), None, guide_params(passes=n))
        p_err = relmse(img)
        rows = []
        for steps in args.headroom_steps:
            g = Guide(ctx, bounds, seed=7)
            passes = max(1, steps // 8)
            render_guided(gs, cam, prm(1, 5), g,
                          guide_params(args.guide_fraction, passes=passes, train_passes=passes, steps_per_pass=8,
                                       batch_samples=1 << 18, learning_rate=1e-2, guide_depth=args.guide_depth,
                                       flags=gflags))
            gimg, gst = render_guided(gs, cam, prm(1, 12), g,
                                      guide_params(args.guide_fraction, passes=n, guide_depth=args.guide_depth))
            g.close()
            e = relmse(gimg)
            rows.append({"train_steps": passes * 8, "relmse": e, "ms": gst.total_ms, "gain": p_err / e})
        print(json.dumps({"metric": "relMSE at equal spp, pre-trained guide vs plain", "unit": "relMSE",
                          "higher_is_better": False,
                          "config": {"workload": workload, "spp": n, "guide_fraction": args.guide_fraction,
                                     "guide_depth": args.guide_depth,
                                     "weights": "absolute" if args.absolute_weights else "pixel-relative",
                                     "target": "BSDF x radiance x cos" if args.product_target else "radiance x cos"},
                          "plain": {"relmse": p_err, "ms": st.total_ms}, "guided": rows}))
        return

    # Passes of k x k samples per pixel (--pass-side k; plain: --plain-pass-side
    # if given); guided passes after training: --late-pass-samples.
    k = args.pass_side
    kp = args.plain_pass_side or k
    plain = []
    for spp in args.spp_list:
        img, st = render_guided(gs, cam, prm(kp, 1000 + spp), None, guide_params(passes=max(1, spp // (kp * kp))))
        plain.append((st.total_ms, relmse(img), st.passes * kp * kp))
    guided = []
    for t, _, spp in plain:
        g = Guide(ctx, bounds, seed=7)
        img, st = render_guided(gs, cam, prm(k, 2000 + spp), g, train_gp(budget_ms=t))
        guided.append((st.total_ms, relmse(img), st.paths // (cam.width * cam.height), st.train_steps, st.train_ms))
        g.close()
    # The network kernels in a trained guide's render, timed per launch.
    g = Guide(ctx, bounds, seed=7)
    _, tst = render_guided(gs, cam, prm(1, 3, _abi.RENDER_TIME_KERNELS), g, train_gp(passes=64))
    _, ist = render_guided(gs, cam, prm(1, 4, _abi.RENDER_TIME_KERNELS), g,
                           guide_params(args.guide_fraction, passes=16))
    g.close()
    f_inf = 2 * (208 * 64 + 64 * 64 + 64 * 64 + 64 * 40)
    f_train = 2 * f_inf + 2 * (64 * 64 + 64 * 64 + 40 * 64)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    inf_tflops = ist.infer_rows * f_inf / (ist.infer_ms * 1e-3) / 1e12 if ist.infer_ms else None
    tr_tflops = tst.train_steps * (1 << 18) * f_train / (tst.train_ms * 1e-3) / 1e12 if tst.train_ms else None
    t_plain = interp_time([(t, e) for t, e, _ in plain], 0.01)
    t_guided = interp_time([(t, e) for t, e, *_ in guided], 0.01)
    line = {"metric": "equal-time relMSE, guided vs plain GPU PT", "unit": "relMSE", "higher_is_better": False,
            "config": {"workload": workload, "reference_spp": ref_spp,
                       "reference_estimator": "guided" if args.ref_guided else "plain",
                       "reference_ms": ref_ms, "guide_fraction": args.guide_fraction,
                       "samples_per_pass": {"plain": kp * kp, "guided_training": k * k,
                                            "guided_late": args.late_pass_samples or k * k},
                       "guide_depth": args.guide_depth, "warmup_steps": args.warmup_steps,
                       "train": "online, Adam lr 1e-2, %d step(s) of 2^18 samples after %s one-spp pass, "
                                "sample weights %s, target %s"
                                % (args.train_steps, "every" if args.train_passes >= 1 << 20
                                   else "each of the first %d" % args.train_passes,
                                   "absolute" if args.absolute_weights else "relative to their pixel",
                                   "BSDF x radiance x cos" if args.product_target else "radiance x cos"),
                       "passes": "inverse-variance weighted (the first, unguided pass seeds the mean)",
                       "training_stream": "second stream, overlapping the next pass" if args.async_train
                       else "the render stream, between passes"},
            "plain": [{"ms": t, "relmse": e, "spp": n} for t, e, n in plain],
            "guided": [{"ms": t, "relmse": e, "spp": n, "train_steps": k, "train_ms": tm}
                       for t, e, n, k, tm in guided],
            "time_to_relmse_0.01_ms": {"plain": t_plain, "guided": t_guided,
                                       "ratio": (t_guided / t_plain) if t_plain and t_guided else None},
            "mlp": {"bound": "tensor", "unit": "TFLOP/s", "peak": tc_peak,
                    "peak_kind": "measured" if "bf16_tflops" in peaks else "fallback",
                    "inference": {"achieved": inf_tflops, "frac": inf_tflops / tc_peak if inf_tflops else None,
                                  "rows": ist.infer_rows, "ms": ist.infer_ms, "flop_per_row": f_inf},
                    "training": {"achieved": tr_tflops, "frac": tr_tflops / tc_peak if tr_tflops else None,
                                 "steps": tst.train_steps, "ms": tst.train_ms, "flop_per_sample": f_train}}}
    if terrain:
        # Throughput at the full 3840 x 2160 view: one-sample passes, plain
        # and with a trained guide.
        del gs
        s.camera = full_cam
        gs = GpuScene(ctx, s)
        fcam = s.camera_struct()
        g = Guide(ctx, scene_bounds(gs), seed=7)
        render_guided(gs, fcam, prm(1, 5), g, train_gp(passes=8))
        _, pst = render_guided(gs, fcam, prm(1, 6), None, guide_params(passes=4))
        _, gst = render_guided(gs, fcam, prm(1, 7), g, guide_params(args.guide_fraction, passes=4))
        g.close()
        line["full_view"] = {"resolution": "%dx%d" % (fcam.width, fcam.height),
                             "plain_paths_per_s": pst.paths / (pst.total_ms * 1e-3),
                             "guided_paths_per_s": gst.paths / (gst.total_ms * 1e-3),
                             "guided_infer_ms_per_pass": gst.infer_ms / max(gst.passes, 1)}
    print(json.dumps(line))


def run_quality(args):
    """relMSE of the benchmark images against 65,536-spp renders accumulated
    in FP64: the Cornell box (256x256, 16 spp, depth 8, reference semantics)
    rendered by the GPU and by the oracle, and the icosphere frame (64 spp)."""
    import numpy as np

    from oracle.binding import OracleScene
    from renderer_gb300 import workloads
    from renderer_gb300.runtime import Context, GpuScene, PerPixelRenderer

    def relmse(x, ref):
        return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))

    def spread(x, ref):
        """Per-pixel relative squared errors: median, and the mean without
        the 0.1 % largest (rare, very bright samples dominate the mean)."""
        e = ((x - ref) ** 2 / (ref ** 2 + 1e-2)).mean(-1).ravel()
        e.sort()
        return {"median": float(np.median(e)), "mean_without_top_0.1pct": float(e[: int(len(e) * 0.999)].mean())}

    ctx = Context(0)
    out = {"metric": "relMSE vs 65,536-spp FP64-accumulated render", "unit": "relMSE", "higher_is_better": False,
           "images": []}
    # Cornell box
    s = workloads.cornell_box(256, 256)
    gs = GpuScene(ctx, s)
    cam = s.camera_struct()

    def gpu(xs, seed, depth, batch=0):
        r = PerPixelRenderer(gs, cam, {"pt-x-samples": xs, "pt-y-samples": xs, "pt-termination-prob": 0.5},
                             seed=seed, max_depth=depth, batch_paths=batch)
        t = time.perf_counter()
        img = r.render()
        return img, time.perf_counter() - t
    ref, tref = gpu(256, 7, 8)
    img, t = gpu(4, 1, 8)
    t0 = time.perf_counter()
    orc = OracleScene(s).render(cam, workloads.cornell_params(8, 3), rng_mode=0)
    tcpu = time.perf_counter() - t0
    out["images"].append({"config": "Cornell box 256x256, 16 spp, depth 8, RR p=0.5 (reference semantics)",
                          "reference": {"spp": 65536, "s": tref},
                          "gpu": {"relmse": relmse(img, ref), "s": t, **spread(img, ref)},
                          "oracle_cpu": {"relmse": relmse(orc["film"], ref), "s": tcpu, **spread(orc["film"], ref)},
                          "gpu_vs_oracle_mean": float(img.mean() / orc["film"].mean())})
    del gs
    # icosphere frame
    s = workloads.icosphere_scene(levels=8, seed=0)
    gs = GpuScene(ctx, s)
    cam = s.camera_struct()
    ref, tref = gpu(256, 7, 12)
    img, t = gpu(8, 1, 12)
    out["images"].append({"config": WORKLOAD, "reference": {"spp": 65536, "s": tref},
                          "gpu": {"relmse": relmse(img, ref), "s": t, **spread(img, ref)}})
    print(json.dumps(out))


CORNELL_WORKLOAD = ("Cornell box (5 diffuse quads, 0.5x0.5 area light of radiance 15, mirror and glass spheres), "
                    "256x256, 4x4 jittered spp, max depth 8, RR p=0.5, reference semantics")


def run_cornell(args):
    """Throughput on the Cornell box (256x256, 16 spp, depth 8): GPU paths/s
    of whole frames (device film, CUDA-event time of gbrt_render_device),
    end to end through gbrt_render (host film), and the oracle's CPU render
    of the same frame on all host cores beside it."""
    import numpy as np

    import renderer_gb300 as rg
    from oracle.binding import OracleScene
    from renderer_gb300 import _abi, workloads
    from renderer_gb300.runtime import Context, GpuScene

    s = workloads.cornell_box(256, 256)
    cam = s.camera_struct()
    ctx = Context(0)
    gs = GpuScene(ctx, s)
    lib = rg.lib()
    import torch
    film = torch.empty(256 * 256 * 3, dtype=torch.float32, device="cuda")
    fsum = torch.empty(256 * 256 * 3, dtype=torch.float64, device="cuda")
    hfilm = np.zeros((256, 256, 3), np.float32)
    prm = workloads.cornell_params(max_depth=8, seed=1)

    def frame_dev():
        st = _abi.Stats()
        rg.check(lib.gbrt_render_device(gs.handle, C.byref(cam), C.byref(prm), C.c_void_p(film.data_ptr()),
                                        C.c_void_p(fsum.data_ptr()), None, C.byref(st)), ctx.handle)
        return st

    for _ in range(args.warmup):
        frame_dev()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    ms, paths, rays, launches = 0.0, 0, 0, 0
    for _ in range(args.steps):
        st = frame_dev()
        ms += st.render_ms
        paths += st.paths
        rays += st.extension_rays + st.shadow_rays
        launches += st.kernel_launches
    t = time.perf_counter()
    for _ in range(args.steps):
        rg.check(lib.gbrt_render(gs.handle, C.byref(cam), C.byref(prm), hfilm.ctypes.data_as(C.c_void_p), None,
                                 None, None, None), ctx.handle)
    e2e_s = time.perf_counter() - t
    clk = clocks.stop()
    del gs
    ctx.close()
    o = OracleScene(s, timing=True)
    t = time.perf_counter()
    r = o.render(cam, prm, rng_mode=0, threads=0)
    cpu_s = time.perf_counter() - t
    line = {"metric": "paths/s (Cornell box)", "value": paths / (ms / 1000.0), "unit": "paths/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": CORNELL_WORKLOAD, "paths_per_step": paths // args.steps,
                       "rays_per_s": rays / (ms / 1000.0),
                       "l2": "scene and path state fit in L2 (a 1M-path frame); whole frames timed back to back"},
            "e2e": {"value": paths / e2e_s, "unit": "paths/s", "h2d_bytes_per_step": C.sizeof(_abi.Camera) +
                    C.sizeof(_abi.RenderParams), "d2h_bytes_per_step": 256 * 256 * 3 * 4},
            "gpu_launches": launches, "clocks": clk,
            "cpu_baseline": {"value": r["paths"] / cpu_s, "unit": "paths/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "the whole frame (%d paths, %.2f s)" % (r["paths"], cpu_s)}}
    print(json.dumps(line))


BATCH_WORKLOAD = ("64 seeded scenes: diffuse 4x3x4 box, 1-3 noise-displaced meshes (log-uniform 10k-2M triangles), "
                  "2-8 spheres, materials uniform over diffuse/mirror/glass 1.5/Blinn 10-500, 1-4 area lights of "
                  "radiance 5-50, 128^2-1024^2 pixels, 4-256 spp, max depth 8, RR p=0.5, reference semantics, "
                  "BVH built on the GPU")


def _batch_scene(i):
    from renderer_gb300 import workloads
    return workloads.batch_scene(i, 0)


def _time_batch(fn, jobs, steps):
    """steps calls of fn(jobs) -> (films, job_ms, stats): device ms, wall ms,
    paths, rays, launches and the mean per-image device times."""
    import numpy as np
    dev_ms, wall_ms, paths, ext, sh, launches, per_image = 0.0, 0.0, 0, 0, 0, 0, []
    for _ in range(steps):
        t = time.perf_counter()
        films, job_ms, st = fn(jobs)
        wall_ms += 1000 * (time.perf_counter() - t)
        dev_ms += st.device_ms
        paths += st.paths
        ext += st.extension_rays
        sh += st.shadow_rays
        launches += st.kernel_launches
        per_image.append(job_ms)
    return dict(dev_ms=dev_ms, wall_ms=wall_ms, paths=paths, ext=ext, sh=sh, launches=launches,
                per_image=np.mean(per_image, 0))


def run_batch(args):
    """Many independent images in one call: aggregate paths/s and per-image
    time over the seeded 64-scene batch. A step is the whole batch; value =
    paths / device span of the batch (films resident), e2e = paths / host wall
    time of the call (films copied to host memory). Default scheduler:
    per-image wavefronts on concurrent streams (gbrt_render_batch); with
    --single-launch the line reports the shared-wavefront, graph-replayed
    batch (gbrt_render_batch_fused) and the stream scheduler beside it."""
    import concurrent.futures as cf
    import multiprocessing as mp

    import numpy as np

    from renderer_gb300 import _abi
    from renderer_gb300.batch import BatchJob, autotune, autotune_fused, render_batch, render_batch_fused
    from renderer_gb300.runtime import Context, GpuScene

    t = time.perf_counter()
    # scene generation (numpy) in spawned workers, before any device work
    with cf.ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as ex:
        scenes = list(ex.map(_batch_scene, range(args.batch_scenes)))
    gen_s = time.perf_counter() - t
    ctx = Context(0)
    t = time.perf_counter()
    gss = [GpuScene(ctx, s) for s, _ in scenes]
    create_s = time.perf_counter() - t
    jobs = [BatchJob(g, s.camera_struct(), p) for g, (s, p) in zip(gss, scenes)]
    t = time.perf_counter()
    S, B = autotune(ctx, jobs) if not args.batch_streams else (args.batch_streams, args.batch_paths or (1 << 22))
    tune_s = time.perf_counter() - t
    fused = None
    if args.single_launch:
        t = time.perf_counter()
        fused = autotune_fused(ctx, jobs)
        fused["autotune_s"] = time.perf_counter() - t
    for _ in range(args.warmup):
        render_batch(ctx, jobs)
        if fused:
            render_batch_fused(ctx, jobs)
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    streams_run = _time_batch(lambda j: render_batch(ctx, j), jobs, args.steps)
    fused_run = _time_batch(lambda j: render_batch_fused(ctx, j), jobs, args.steps) if fused else None
    clk = clocks.stop()
    run = fused_run if fused else streams_run
    dev_ms, wall_ms, paths, ext, sh, launches = (run[k] for k in ("dev_ms", "wall_ms", "paths", "ext", "sh",
                                                                  "launches"))
    per_image = run["per_image"]
    tri = [s.n_tri() for s, _ in scenes]
    spp = [p.x_samples * p.y_samples for _, p in scenes]
    res = [s.camera["width"] for s, _ in scenes]
    d2h = sum(r * r * 3 * 4 for r in res)
    h2d = len(jobs) * C.sizeof(_abi.BatchJob)
    depth = max(p.max_depth for _, p in scenes)
    line = {"metric": "paths/s (batch)", "value": paths / (dev_ms / 1000.0), "unit": "paths/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": BATCH_WORKLOAD, "scenes": len(jobs), "paths_per_step": paths // args.steps,
                       "triangles_total": int(sum(tri)), "triangles_min": int(min(tri)),
                       "triangles_max": int(max(tri)), "resolutions": {str(r): res.count(r) for r in sorted(set(res))},
                       "spp": {str(v): spp.count(v) for v in sorted(set(spp))},
                       "streams": S, "batch_paths": B, "autotune_s": tune_s, "scene_generation_s": gen_s,
                       "scene_create_s": create_s,
                       "l2": "inputs larger than L2 (33M triangles over 64 scenes, path state per stream > 129 MB)",
                       "per_image_ms": {"mean_wall": wall_ms / args.steps / len(jobs),
                                        "device_median": float(np.median(per_image)),
                                        "device_max": float(np.max(per_image)),
                                        "device_min": float(np.min(per_image))},
                       "extension_rays_per_path": ext / max(paths, 1), "shadow_rays_per_path": sh / max(paths, 1),
                       "max_depth": depth,
                       "scheduler": "single launch (shared wavefronts, CUDA graph per wavefront)" if fused
                       else "streams (one wavefront pipeline per image)"},
            "e2e": {"value": paths / (wall_ms / 1000.0), "unit": "paths/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clk}
    if fused:
        def summary(r):
            return {"paths_per_s": r["paths"] / (r["dev_ms"] / 1000.0),
                    "e2e_paths_per_s": r["paths"] / (r["wall_ms"] / 1000.0),
                    "ms_per_step": r["dev_ms"] / args.steps, "kernel_launches_per_step": r["launches"] // args.steps,
                    "per_image_ms_median": float(np.median(r["per_image"])),
                    "per_image_ms_max": float(np.max(r["per_image"]))}
        line["config"]["designs"] = {"single_launch": dict(summary(fused_run), **fused),
                                     "streams": dict(summary(streams_run), streams=S, batch_paths=B)}
    print(json.dumps(line))


INSTANCED_WORKLOAD = ("8 instances of one 4,000,000-triangle noise-displaced terrain (two-level BVH), 200 spheres "
                      "(diffuse/mirror/glass/Blinn), 2048x1024 lat-long sky with a sun; 16 seeded views at "
                      "3840x2160, 1 spp each, max depth 16, RR p=0.5, physical semantics")


def guided_views(args, ctx, gs, cams):
    """The 16 views guided by one network trained online on all of them (2
    one-sample training passes per view, 4 Adam steps of 2^18 samples after
    each, product target), then one guided sample per pixel of every view
    with the trained guide: aggregate paths/s over the views' device time,
    and the inference rate of the network against the dense-BF16 peak."""
    from renderer_gb300 import _abi
    from renderer_gb300.guiding import Guide, guide_params, render_guided, scene_bounds
    from renderer_gb300.scene import SceneData, render_params

    def cam(c):
        sc = SceneData()
        sc.camera = c
        return sc.camera_struct()

    def prm(seed, flags=0):
        return render_params(1, 1, 0.5, 16, seed, semantics=_abi.SEM_PHYSICAL, flags=flags)

    g = Guide(ctx, scene_bounds(gs), seed=7)
    t = time.perf_counter()
    steps = 0
    for i, c in enumerate(cams):
        _, st = render_guided(gs, cam(c), prm(300 + i), g,
                              guide_params(0.5, passes=2, train_passes=2, steps_per_pass=4, batch_samples=1 << 18,
                                           learning_rate=1e-2, flags=_abi.GUIDE_PRODUCT))
        steps += st.train_steps
    train_s = time.perf_counter() - t
    ms, paths, ext = 0.0, 0, 0
    for step in range(args.steps):
        for i, c in enumerate(cams):
            _, st = render_guided(gs, cam(c), prm(400 + 16 * step + i), g, guide_params(0.5, passes=1))
            ms += st.total_ms
            paths += st.paths
            ext += st.extension_rays
    rows, inf_ms = 0, 0.0
    for i, c in enumerate(cams):
        _, st = render_guided(gs, cam(c), prm(500 + i, _abi.RENDER_TIME_KERNELS), g, guide_params(0.5, passes=1))
        rows += st.infer_rows
        inf_ms += st.infer_ms
    g.close()
    f_inf = 2 * (208 * 64 + 64 * 64 + 64 * 64 + 64 * 40)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    tflops = rows * f_inf / (inf_ms * 1e-3) / 1e12 if inf_ms else None
    return {"views": len(cams), "resolution": "%dx%d" % (cams[0]["width"], cams[0]["height"]),
            "paths_per_s": paths / (ms * 1e-3), "ms_per_step": ms / args.steps,
            "extension_rays_per_path": ext / max(paths, 1),
            "train": "online on all views: %d Adam steps of 2^18 samples (product target) in %.1f s" % (steps, train_s),
            "mlp": {"bound": "tensor", "unit": "TFLOP/s", "achieved": tflops, "peak": tc_peak,
                    "peak_kind": "measured" if "bf16_tflops" in peaks else "fallback",
                    "frac": tflops / tc_peak if tflops else None, "rows": rows, "ms": inf_ms}}


def run_instanced(args):
    """The instanced-terrain scene: 16 views of 3840 x 2160 at one sample per
    pixel in one gbrt_render_batch call (a step = all 16 images). value =
    paths / device span; e2e = paths / host wall time of the call, the 16
    films (1.6 GB) copied to host memory. --single-launch renders the 16
    views in one gbrt_render_batch_fused call instead (every kernel launch
    serves all views, one CUDA graph per wavefront, autotuned schedule) and
    reports the stream scheduler beside it. --compare-flat also renders the
    same views of the scene with every instance flattened into one tree."""
    import numpy as np

    from renderer_gb300 import _abi, workloads
    from renderer_gb300.batch import BatchJob, autotune_fused, render_batch, render_batch_fused
    from renderer_gb300.runtime import Context, GpuScene
    from renderer_gb300.scene import SceneData, render_params

    t = time.perf_counter()
    s, cams = workloads.terrain_instances(seed=0, nx=args.terrain_nx, nz=args.terrain_nx // 2)
    gen_s = time.perf_counter() - t
    ctx = Context(0)
    t = time.perf_counter()
    gs = GpuScene(ctx, s)
    create_s = time.perf_counter() - t
    info = gs.info()

    def measure(scene, tag, fused=False):
        jobs = []
        for i, c in enumerate(cams):
            sc = SceneData()
            sc.camera = c
            jobs.append(BatchJob(scene, sc.camera_struct(),
                                 render_params(1, 1, 0.5, 16, 100 + i, semantics=_abi.SEM_PHYSICAL)))
        tuned = None
        if fused:
            t0 = time.perf_counter()
            tuned = autotune_fused(ctx, jobs)
            tuned["autotune_s"] = time.perf_counter() - t0
            call = lambda: render_batch_fused(ctx, jobs)  # noqa: E731
        else:
            call = lambda: render_batch(ctx, jobs, streams=4)  # noqa: E731
        for _ in range(args.warmup):
            call()
        clocks = ClockSampler(0)
        clocks.start()
        time.sleep(0.3)
        dev, wall, paths, ext, sh = 0.0, 0.0, 0, 0, 0
        for _ in range(args.steps):
            t0 = time.perf_counter()
            films, _, st = call()
            wall += time.perf_counter() - t0
            dev += st.device_ms / 1000.0
            paths += st.paths
            ext += st.extension_rays
            sh += st.shadow_rays
        clk = clocks.stop()
        return {"value": paths / dev, "e2e": paths / wall, "ms_per_step": 1000 * dev / args.steps,
                "rays_per_s": (ext + sh) / dev, "extension_rays_per_path": ext / paths,
                "shadow_rays_per_path": sh / paths, "clocks": clk, "film_mean": float(films[0].mean()),
                "launches": st.kernel_launches, "schedule": tuned}

    r = measure(gs, "two-level")
    designs = None
    if args.single_launch:
        rf = measure(gs, "two-level", fused=True)
        designs = {"single_launch": {"paths_per_s": rf["value"], "e2e_paths_per_s": rf["e2e"],
                                     "ms_per_step": rf["ms_per_step"], "kernel_launches_per_step": rf["launches"],
                                     "film_mean_view0": rf["film_mean"], **rf["schedule"]},
                   "streams": {"paths_per_s": r["value"], "e2e_paths_per_s": r["e2e"],
                               "ms_per_step": r["ms_per_step"], "kernel_launches_per_step": r["launches"],
                               "film_mean_view0": r["film_mean"], "streams": 4}}
        r = rf
    tri = len(s.meshes[0]["pos"]) * len(s.instances)
    line = {"metric": "paths/s (instanced terrain, 16 views)", "value": r["value"], "unit": "paths/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": INSTANCED_WORKLOAD, "paths_per_step": 16 * cams[0]["width"] * cams[0]["height"],
                       "mesh_triangles": len(s.meshes[0]["pos"]), "instanced_triangles": tri,
                       "scene_generation_s": gen_s, "scene_create_s": create_s, "bvh_nodes": info["nodes"],
                       "rays_per_s": r["rays_per_s"], "extension_rays_per_path": r["extension_rays_per_path"],
                       "shadow_rays_per_path": r["shadow_rays_per_path"],
                       "l2": "inputs larger than L2 (mesh 4M triangles, path state per stream > 129 MB)",
                       "scheduler": "single launch (shared wavefronts, CUDA graph per wavefront)" if designs
                       else "streams (one wavefront pipeline per view)"},
            "e2e": {"value": r["e2e"], "unit": "paths/s", "h2d_bytes_per_step": 16 * C.sizeof(_abi.BatchJob),
                    "d2h_bytes_per_step": 16 * cams[0]["width"] * cams[0]["height"] * 12},
            "gpu_launches": r["launches"] * args.steps, "clocks": r["clocks"]}
    if designs:
        line["config"]["designs"] = designs
    if args.guided_views:
        line["guided_views"] = guided_views(args, ctx, gs, cams)
    if args.compare_flat:
        del gs
        f = SceneData(materials=s.materials, spheres=s.spheres, lights=s.lights, env=s.env, env_mapping=s.env_mapping,
                      camera=s.camera)
        P, N = [], []
        m = s.meshes[0]
        for M, _ in s.instances:
            A = np.asarray(M)[:, :3].astype(np.float32)
            tt = np.asarray(M)[:, 3].astype(np.float32)
            P.append((m["pos"].reshape(-1, 3) @ A.T + tt).reshape(-1, 9))
            nn = m["nrm"].reshape(-1, 3) @ np.linalg.inv(A.astype(np.float64))
            N.append((nn / np.linalg.norm(nn, axis=1, keepdims=True)).astype(np.float32).reshape(-1, 9))
        f.tri_pos = np.concatenate(P)
        f.tri_nrm = np.concatenate(N)
        f.tri_mat = np.concatenate([m["mat"]] * len(s.instances))
        del P, N
        t = time.perf_counter()
        gf = GpuScene(ctx, f)
        fc = time.perf_counter() - t
        rf = measure(gf, "flat")
        line["config"]["flattened"] = {"value": rf["value"], "scene_create_s": fc, "bvh_nodes": gf.info()["nodes"],
                                       "film_mean": rf["film_mean"], "two_level_film_mean": r["film_mean"]}
    print(json.dumps(line))


def run_chains(args):
    """The Markov-chain renderers on the Cornell box (256 x 256, max depth 5,
    the renderer's defaults: Metropolis with 16 mutations per pixel, 10,000
    bootstrap samples, large steps 0.1, termination 0.5; energy
    redistribution with 100 mutations per chain and 2 x 2 initial samples per
    pixel): paths traced per second of device time for several chain counts,
    beside the oracle's restatement on the host cores (one chain per thread,
    as the renderer runs)."""
    import numpy as np

    from oracle.binding import OracleScene
    from renderer_gb300 import workloads
    from renderer_gb300.chains import EnergyRedistributionRenderer, MetropolisRenderer, erpt_params, mlt_params
    from renderer_gb300.runtime import Context, GpuScene
    from renderer_gb300.scene import render_params

    s = workloads.cornell_box(256, 256)
    ctx = Context(0)
    gs = GpuScene(ctx, s)
    out = {"metric": "paths/s (Markov-chain renderers)", "unit": "paths/s", "higher_is_better": True,
           "config": {"workload": "Cornell box 256x256, max depth 5, reference semantics"}, "mlt": [], "erpt": []}
    for chains in args.mlt_chains:
        r = MetropolisRenderer(gs, seed=1, max_depth=5, chains=chains)
        for _ in range(args.warmup):
            r.render()
        ms, paths = 0.0, 0
        for _ in range(args.steps):
            r.render()
            ms += r.stats.render_ms
            paths += r.stats.paths
        st = r.stats
        out["mlt"].append({"chains": st.chains, "mutations_per_chain": st.mutations // st.chains,
                           "value": paths / (ms / 1000.0), "ms_per_image": ms / args.steps,
                           "acceptance": st.accepted / st.mutations, "kernel_launches": st.kernel_launches})
    r = EnergyRedistributionRenderer(gs, seed=1, max_depth=5)
    for _ in range(args.warmup):
        r.render()
    ms, paths = 0.0, 0
    for _ in range(args.steps):
        r.render()
        ms += r.stats.render_ms
        paths += r.stats.paths
    st = r.stats
    out["erpt"].append({"chains": st.chains, "value": paths / (ms / 1000.0), "ms_per_image": ms / args.steps,
                        "acceptance": st.accepted / st.mutations, "kernel_launches": st.kernel_launches})
    del gs
    ctx.close()
    if not args.no_cpu_baseline:
        o = OracleScene(s, timing=True)
        cam = s.camera_struct()
        t = time.perf_counter()
        rr = o.render_mlt(cam, render_params(1, 1, 0.0, 5, 1), mlt_params(1, 10000), chains=64)
        dt = time.perf_counter() - t
        out["cpu_baseline_mlt"] = {"value": rr["paths"] / dt, "unit": "paths/s", "cores": 1, "kind": "port",
                                   "sample": "1 mutation per pixel over 64 chains (%d paths, %.1f s)"
                                   % (rr["paths"], dt)}
        t = time.perf_counter()
        re_ = o.render_erpt(cam, render_params(1, 1, 0.0, 5, 1), erpt_params(4, 1, 1))
        dt = time.perf_counter() - t
        out["cpu_baseline_erpt"] = {"value": re_["paths"] / dt, "unit": "paths/s", "cores": 1, "kind": "port",
                                    "sample": "4 mutations per chain, 1 initial sample per pixel (%d paths, %.1f s)"
                                    % (re_["paths"], dt)}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-rows", type=int, default=128, help="rows in the CPU-baseline sample (about 11 s on 16 cores)")
    ap.add_argument("--reference-rows", type=int, default=32, help="rows per step of --impl reference")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-paths", type=int, default=0)
    ap.add_argument("--profile", action="store_true",
                    help="for ncu: one untimed frame, then one frame, nothing else")
    ap.add_argument("--gpu-build", action="store_true",
                    help="build the BVH on the GPU (GBRT_SCENE_GPU_BUILD) instead of the host's binned SAH")
    ap.add_argument("--guided", action="store_true",
                    help="equal-time relMSE of neural path guiding against plain path tracing (two rooms)")
    ap.add_argument("--ref-spp", type=int, default=65536)
    ap.add_argument("--guided-scene", default="rooms", choices=["rooms", "terrain"],
                    help="--guided on the two rooms or on view 0 of the instanced terrain")
    ap.add_argument("--ref-guided", action="store_true",
                    help="--guided: render the reference with a guide trained online (unbiased as well)")
    ap.add_argument("--guided-width", type=int, default=960)
    ap.add_argument("--guided-height", type=int, default=540)
    ap.add_argument("--ref-cache", default="", help="npz file holding (or receiving) the reference render")
    ap.add_argument("--spp-list", type=lambda x: [int(v) for v in x.split(",")], default=SPP_DEFAULT)
    ap.add_argument("--guide-fraction", type=float, default=0.5)
    ap.add_argument("--guide-depth", type=int, default=0, help="guide vertices i < this only (0: all)")
    ap.add_argument("--warmup-steps", type=int, default=0, help="BSDF-only passes until this many training steps")
    ap.add_argument("--absolute-weights", action="store_true",
                    help="--guided: training weights not relative to the sample's pixel")
    ap.add_argument("--train-passes", type=int, default=1 << 30, help="passes that train (default: all)")
    ap.add_argument("--async-train", action="store_true",
                    help="with --guided: Adam steps on a second stream, overlapping the next pass")
    ap.add_argument("--product-target", action="store_true",
                    help="--guided: the guide learns BSDF x incident radiance x cos (GBRT_GUIDE_PRODUCT)")
    ap.add_argument("--tuned", action="store_true",
                    help="--guided with the best settings found on the two rooms: the product target, sample "
                         "weights not relative to their pixel, 16 Adam steps after each of the first 32 passes, "
                         "BSDF-only passes for the first 256 steps, passes of 16 samples after training; plain "
                         "at its fastest, 64 samples per pass")
    ap.add_argument("--train-steps", type=int, default=1, help="Adam steps of 2^18 samples after a training pass")
    ap.add_argument("--pass-side", type=int, default=1,
                    help="--guided: k x k samples per pixel per pass, for the plain and the guided renderer")
    ap.add_argument("--plain-pass-side", type=int, default=0,
                    help="--guided: k x k samples per pixel per pass of the plain renderer (0: --pass-side)")
    ap.add_argument("--late-pass-samples", type=int, default=0,
                    help="--guided: samples per pixel of the guided passes after training (0: as in training)")
    ap.add_argument("--headroom", action="store_true",
                    help="--guided: relMSE at equal spp of guides pre-trained untimed for --headroom-steps steps")
    ap.add_argument("--headroom-steps", type=lambda x: [int(v) for v in x.split(",")], default=[256, 2048, 8192])
    ap.add_argument("--headroom-spp", type=int, default=128)
    ap.add_argument("--quality", action="store_true",
                    help="relMSE of the Cornell box and icosphere images against 65,536-spp renders")
    ap.add_argument("--batch", action="store_true",
                    help="aggregate paths/s of the seeded 64-scene batch through gbrt_render_batch")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--cornell", action="store_true", help="throughput on the Cornell box (256x256, 16 spp, depth 8)")
    ap.add_argument("--batch-streams", type=int, default=0, help="streams for --batch (0: autotune)")
    ap.add_argument("--single-launch", action="store_true",
                    help="with --batch: the shared-wavefront batch under CUDA graphs, beside the stream scheduler")
    ap.add_argument("--instanced", action="store_true",
                    help="16 views of the instanced-terrain scene (two-level BVH) through gbrt_render_batch")
    ap.add_argument("--terrain-nx", type=int, default=2000, help="terrain quads along x (2000: 4M triangles)")
    ap.add_argument("--compare-flat", action="store_true", help="with --instanced: also the flattened scene")
    ap.add_argument("--guided-views", action="store_true",
                    help="with --instanced: also the 16 views guided by one network trained on them")
    ap.add_argument("--chains", action="store_true",
                    help="paths/s of the Metropolis and energy-redistribution renderers (Cornell box)")
    ap.add_argument("--mlt-chains", type=lambda x: [int(v) for v in x.split(",")], default=[0, 4096, 1 << 20],
                    help="chain counts for --chains (0: the library's default)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.tuned:
        args.absolute_weights, args.product_target = True, True
        args.train_steps, args.train_passes, args.warmup_steps = 16, 32, 256
        # guided passes of 16 samples once training is over; plain at its
        # fastest pass size (64 samples per pass), so spp from 64 up
        args.late_pass_samples = args.late_pass_samples or 16
        args.plain_pass_side = args.plain_pass_side or 8
        if args.spp_list == SPP_DEFAULT:
            args.spp_list = [64, 128, 256, 512, 1024]
    if args.chains:
        run_chains(args)
        return
    if args.instanced:
        run_instanced(args)
        return
    if args.cornell:
        run_cornell(args)
        return
    if args.batch:
        run_batch(args)
        return
    if args.quality:
        run_quality(args)
        return
    if args.guided:
        run_guided(args)
        return
    ws, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank, dist)
        return

    import numpy as np
    import torch

    import renderer_gb300 as rg
    from renderer_gb300 import _abi, workloads
    from renderer_gb300.runtime import Context, GpuScene

    torch.cuda.set_device(local)
    s = workloads.icosphere_scene(levels=8, seed=0)
    if args.gpu_build:
        s.flags = _abi.SCENE_GPU_BUILD
    cam = s.camera_struct()
    H, W = cam.height, cam.width
    ctx = Context(local)
    gs = GpuScene(ctx, s)
    info = gs.info()
    lib = rg.lib()

    film = torch.empty(H * W * 3, dtype=torch.float32, device="cuda")
    fsum = torch.empty(H * W * 3, dtype=torch.float64, device="cuda")
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def render_dev(flags, stats):
        p = workloads.icosphere_params()
        p.flags = flags
        p.batch_paths = args.batch_paths
        rg.check(lib.gbrt_render_device(gs.handle, C.byref(cam), C.byref(p), ptr(film), ptr(fsum), None,
                                        C.byref(stats)), ctx.handle)

    if args.profile:
        for _ in range(2):
            st = _abi.Stats()
            render_dev(0, st)
        torch.cuda.synchronize()
        print(json.dumps({"profile_frames": 2, "paths": st.paths, "render_ms": st.render_ms,
                          "launches_per_frame": st.kernel_launches, "extension_rays": st.extension_rays,
                          "shadow_rays": st.shadow_rays,
                          "batch_paths": args.batch_paths or 67108864}))
        return

    # Traversal work of this workload (untimed pass with counters).
    cs = _abi.Stats()
    render_dev(_abi.RENDER_COUNT_TRAVERSAL, cs)
    n_node = cs.nodes_closest / max(cs.extension_rays, 1)
    n_prim = cs.prims_closest / max(cs.extension_rays, 1)
    # Algorithmic bytes per ray: ray + hit + 64 B per node visit + 48 B per
    # primitive test. Beside it, what the kernel fetches per visit of its
    # 4-wide node: 7 x 16 B (six box planes + child references).
    bytes_per_ray = 32 + 16 + 64 * n_node + 48 * n_prim
    fetched_per_ray = 32 + 16 + 112 * n_node + 48 * n_prim

    for _ in range(args.warmup):
        render_dev(0, _abi.Stats())
    clocks = ClockSampler(local)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    tot = dict(ms=0.0, ext_ms=0.0, shade_ms=0.0, shadow_ms=0.0, ext_launch=0, ext_rays=0, sh_rays=0, paths=0,
               launches=0)
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        st = _abi.Stats()
        render_dev(_abi.RENDER_TIME_KERNELS, st)
        tot["ms"] += st.render_ms
        tot["ext_ms"] += st.extend_ms
        tot["shade_ms"] += st.shade_ms
        tot["shadow_ms"] += st.shadow_ms
        tot["ext_launch"] += st.extend_launches
        tot["ext_rays"] += st.extension_rays
        tot["sh_rays"] += st.shadow_rays
        tot["paths"] += st.paths
        tot["launches"] += st.kernel_launches
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    barrier(dist)
    clk = clocks.stop()
    ms = max_over_ranks(tot["ms"], dist)
    value = tot["paths"] * ws / (ms / 1000.0)

    # End to end through the C ABI with host buffers (film back every frame).
    hfilm = np.zeros((H, W, 3), np.float32)
    p = workloads.icosphere_params()
    p.batch_paths = args.batch_paths
    e2e_s = 0.0
    e2e_paths = 0
    for i in range(args.warmup + args.steps):
        st = _abi.Stats()
        barrier(dist)
        t0 = time.perf_counter()
        rg.check(lib.gbrt_render(gs.handle, C.byref(cam), C.byref(p), hfilm.ctypes.data_as(C.c_void_p), None, None,
                                 None, C.byref(st)), ctx.handle)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_s += dt
            e2e_paths += st.paths
    e2e_s = max_over_ranks(e2e_s, dist)
    e2e = e2e_paths * ws / e2e_s

    peak, peak_kind = measured_peaks()
    ext_s = tot["ext_ms"] / 1000.0
    achieved = tot["ext_rays"] * bytes_per_ray / ext_s / 1e9
    launches = max(tot["ext_launch"], 1)
    avg_launch_s = ext_s / launches
    # DRAM and L2 bytes of an average launch: the committed capture's bytes
    # per camera ray and per bounce ray times this run's ray counts.
    tr = extend_traffic()
    traffic = l2_traffic = dram_frac = None
    if tr is not None:
        n_cam, n_bounce = tot["paths"], tot["ext_rays"] - tot["paths"]
        traffic = (tr["camera"]["dram_bytes_per_ray"] * n_cam
                   + tr["bounce"]["dram_bytes_per_ray"] * n_bounce) / launches
        l2_traffic = (tr["camera"]["l2_bytes_per_ray"] * n_cam
                      + tr["bounce"]["l2_bytes_per_ray"] * n_bounce) / launches
        dram_frac = traffic / avg_launch_s / 1e9 / peak
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind + " (copy bandwidth)",
                "traffic": traffic, "l2_traffic": l2_traffic,
                "traffic_source": None if tr is None else
                "ncu capture of a whole frame (profiles/k_extend_icosphere_traffic.json), per camera and per "
                "bounce ray, scaled by this run's ray counts",
                "dram_frac": dram_frac,
                "kernel": "k_extend (closest-hit BVH traversal)",
                "bytes_per_ray": bytes_per_ray,
                "bytes_per_ray_formula": "32 (ray) + 16 (hit) + 64 x node visits + 48 x primitive tests",
                "nodes_per_ray": n_node, "prims_per_ray": n_prim,
                "fetched_bytes_per_ray": fetched_per_ray,
                "frac_fetched": tot["ext_rays"] * fetched_per_ray / ext_s / 1e9 / peak,
                "bound_note": "issue- and divergence-bound, not bandwidth-bound: nodes and records come mostly "
                              "from L1/L2 (dram_frac is what DRAM carries); ncu: 72-75 % issue-active, 21 of 32 "
                              "lanes active on camera rays and 9 on bounces (profiles/k_extend_icosphere.md)",
                "launches": tot["ext_launch"], "avg_launch_ms": 1000.0 * avg_launch_s,
                "share_of_render": tot["ext_ms"] / max(tot["ms"], 1e-9)}

    line = {"metric": "paths/s", "value": value, "unit": "paths/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "paths_per_step": tot["paths"] // args.steps,
                       "bvh_build": "gpu (linear BVH)" if args.gpu_build else "host (binned SAH)",
                       "l2": "inputs larger than L2 (scene ~240 MB, path state ~20 GB per wavefront)",
                       "scene_build_ms": info["build_ms"], "bvh_nodes": info["nodes"],
                       "bvh_max_depth": info["max_depth"], "wall_s_timed": wall,
                       "rays_per_s": (tot["ext_rays"] + tot["sh_rays"]) * ws / (ms / 1000.0),
                       "kernel_ms_per_step": {"extend": tot["ext_ms"] / args.steps,
                                              "shade": tot["shade_ms"] / args.steps,
                                              "shadow": tot["shadow_ms"] / args.steps},
                       "extension_rays_per_path": tot["ext_rays"] / max(tot["paths"], 1),
                       "shadow_rays_per_path": tot["sh_rays"] / max(tot["paths"], 1)},
            "roofline": roofline,
            "e2e": {"value": e2e, "unit": "paths/s", "h2d_bytes_per_step": C.sizeof(_abi.Camera) +
                    C.sizeof(_abi.RenderParams), "d2h_bytes_per_step": H * W * 3 * 4},
            "gpu_launches": tot["launches"], "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        del gs
        ctx.close()
        rate, n, dt, cores = cpu_baseline(s, cam, workloads.icosphere_params(), args.cpu_rows)
        line["cpu_baseline"] = {"value": rate, "unit": "paths/s", "cores": cores, "kind": "port",
                                "sample": "%d evenly spaced rows (%d paths, %.1f s) of the same frame"
                                % (args.cpu_rows, n, dt)}
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
