#!/usr/bin/env python3
"""Benchmark of the render hot path through the C ABI (libcrg.so).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl crg|reference]
                    [--workload batch|box|displaced|soup|inverse]

Workloads (seeded synthetic inputs; no external data):
  batch      (default) 64 views drawn from the box and displaced scenes with
             resolutions in {128^2 .. 1920x1080} and spp in {16, 64, 256}
             (4.73G samples): the wavefront form renders the whole batch in one
             graph launch per step; the megakernel renders the same views one
             crg_render call each.  Both produce bit-identical films, so equal
             RMSE holds by construction.  Metric: Msamples/s (wavefront).
  box        the 36-triangle box scene, 512x512, 64 spp, 8 segments, RR from 3,
             extended estimator, megakernel.  Metric: Msamples/s.
  displaced  the displaced icosphere (4,196,562 triangles), 1920x1080, 16 of the
             256 spp per step (a frame is 16 steps), depth 16, megakernel.
  soup       1,048,576-triangle soup, 16,777,216 closest-hit rays.  Mrays/s.
  inverse    inverse rendering of the box scene (34 per-triangle albedos + light
             radiance), 256x256: a step is one forward (32 spp), the L2 loss
             against a 4096-spp target and one path-replay backward (32 spp).
             Msamples/s over forward + backward samples; also reports the
             backward/forward time ratio, central-FD agreement (h = 1e-3,
             common random numbers) and a 200-step Adam run (lr 0.02).

`value` is device-timed (CUDA events on the launching stream; inputs resident;
L2 flushed by a 256 MiB write between steps, outside the events).  `e2e` runs
the same step through the public C ABI from pinned host buffers (scene upload,
BVH build, render, film download).  `time_to_rmse` (batch and box workloads):
time for the box configuration to reach RMSE <= 1e-2 against an FP64
16384-spp image.  --impl reference times the CPU oracle (the C++ restatement
of the reference integrator; Embree cannot be built here) on all host cores on
a bounded sample.  Multi-GPU runs are independent replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BOX = dict(width=512, height=512, spp=64, max_bounces=8, rr_depth=3, mode=1, seed=1)
L2_NOTE = "flushed between steps (256 MiB write, outside the timed events)"


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.stop = threading.Event()
        self.th = None

    def _run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5).stdout
                self.rows.append([x.strip() for x in out.strip().split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.th = threading.Thread(target=self._run, daemon=True)
        self.th.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.th.join(timeout=10)

    def summary(self):
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[0]) for r in self.rows if r and num(r[0]) is not None]
        mx = [num(r[1]) for r in self.rows if len(r) > 1 and num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


POST = dict(width=3840, height=2160)
# leaf sizes the autotuner tries per scene (bit mask of 1 << leaf_max)
LEAVES = (1 << 1) | (1 << 2) | (1 << 3)
# (width, treelet, leaf_max) fastest for the megakernel in a GB300 sweep of width {4, 8} x leaf {1, 2, 3}
# x treelet rounds {3, 6}: box 616-623 Msamples/s at width 4 (592 at 8), displaced 655 at width 4 leaf 1
# (579 at width 8 leaf 3)
MEGA_BVH = {"box": (4, 1, 2), "displaced": (4, 1, 1)}


def post_settings_full(api):
    """Every post-processing pass on: bloom (threshold 0.7, strength 1), gray scale off,
    Uncharted tone curve with exposure 1.5 and gamma 2.2, every pixel covered."""
    return api.post_settings(bloom=1, tonemapping=1, tonemap_type=3, exposure=1.5, mode=1)


def post_image(w, h):
    r = np.random.default_rng(7)
    img = r.gamma(0.6, 0.8, (h, w, 4)).astype(np.float32)
    img[..., 3] = 1.0
    return img


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) from ncu captures on a GB300:
#   one wavefront frame, per sample: box scene 512x512x64 1,720 B; displaced scene
#   1920x1080x16 (path pool 4,194,304) 1,097 B;
#   k_intersect on the soup, per launch of 16,777,216 closest-hit rays: 923.3 MB.
TRAFFIC_PER_SAMPLE = {"box": 1720.0, "displaced": 1097.0}
TRAFFIC_SOUP_LAUNCH = 923.3e6


# DRAM bytes per traversed ray (read + write) of the extend kernel, from the displaced-scene
# iteration capture (profiles/wavefront_displaced_iteration_full.md, build C: 811 MB over one
# full-queue iteration of a 4,194,304-path pool, one ray per path)
DRAM_PER_RAY = {"extend": 811.3e6 / 4194304}


def traffic_dominant(out, stage):
    """DRAM traffic of one frame's launches of a traversal stage: ncu bytes per ray x the frame's rays."""
    w = out.get("work", {})
    rays = w.get("segments" if stage == "extend" else "shadow_rays")
    return DRAM_PER_RAY[stage] * rays if rays and stage in DRAM_PER_RAY else None


def traffic_estimate(workload, out, units):
    """DRAM traffic per step from the ncu captures above, or None; the batch is
    scaled per scene by its samples (the per-sample traffic of a frame grows in
    proportion to its samples once the path pool exceeds L2)."""
    if workload == "soup":
        return TRAFFIC_SOUP_LAUNCH, "ncu capture of the same launch"
    if workload == "batch" and "scene_samples" in out:
        t = sum(TRAFFIC_PER_SAMPLE[k] * v for k, v in out["scene_samples"].items())
        return t, "per-sample traffic of one wavefront frame of each scene (ncu), scaled by the batch's samples per scene"
    if workload in ("box", "displaced") and out.get("form") == "wavefront":
        return TRAFFIC_PER_SAMPLE[workload] * units, "per-sample traffic of one wavefront frame (ncu), times the samples"
    return None, None


# L2 hit rates (lts__t_sector_hit_rate) of the traversal kernels from ncu captures on a GB300
# (profiles/wavefront_displaced_iteration_full.md, build C; profiles/k_intersect_soup_full.md)
L2_HIT = {"extend": 0.671, "shadow": 0.671, "soup_closest": 0.880, "soup_any": 0.860}


def stage_roofline(tuned, work, sh_work, stages, node_bytes, peak):
    """Roofline of the traversal stages of a wavefront frame and the time share of every stage.
    Algorithmic bytes of a traversal stage: 48 B per ray (32 B ray in, 16 B hit or flag out) plus
    node_bytes per wide node visited and 48 B per triangle tested, from the instrumented frame; its
    time is the sum of its launches' CUDA-event durations over a frame of the host-driven loop."""
    fuse = tuned.get("fuse", 1) or 1
    ext_bytes = (work["segments"] * 48 + (work["nodes_visited"] - sh_work["shadow_nodes"]) * node_bytes
                 + (work["tris_tested"] - sh_work["shadow_tris"]) * 48)
    sh_bytes = work["shadow_rays"] * 48 + sh_work["shadow_nodes"] * node_bytes + sh_work["shadow_tris"] * 48
    # which launches carry which traversal: fuse 1 split stages, 2 shadow test inside shade, 3 all inside shade
    carried = {1: {"extend": ext_bytes, "shadow": sh_bytes}, 2: {"extend": ext_bytes, "shade": sh_bytes},
               3: {"shade": ext_bytes + sh_bytes}}[fuse]
    ms = {"extend": stages["extend_ms"], "shade": stages["shade_ms"], "shadow": stages["shadow_ms"],
          "control_resolve_generate": stages["other_ms"]}
    total = sum(ms.values())
    refill = tuned.get("refill", 16)
    kernels = {"extend": "k_wf_extend_dyn" if refill else "k_wf_extend", "shade": "k_wf_shade",
               "shadow": "k_wf_shadow_dyn" if refill else "k_wf_shadow"}
    rows = {}
    for k, b in carried.items():
        if ms[k] > 0:
            gbs = b / (ms[k] / 1e3) / 1e9
            rows[k] = {"kernel": kernels[k], "algorithmic_bytes": int(b), "ms": ms[k], "achieved_gbs": gbs,
                       "frac": gbs / peak}
    dom = max(rows, key=lambda k: ms[k]) if rows else None
    return {"ms": ms, "share": {k: v / total for k, v in ms.items()} if total else {}, "frame_ms_host_loop": total,
            "iterations": stages["iterations"], "traversal": rows, "dominant": dom,
            "how": "one frame through the host-driven loop (host_loop 2) with CUDA events around every stage; "
                   "traversal work from an instrumented frame"}


def workload_config(w, form="megakernel"):
    if w == "post":
        return {"workload": "post-processing of a 3840x2160 RGBA32F image: bloom threshold + 10 separable 15-tap "
                            "blur passes + composite with the Uncharted tone curve (every pixel covered)",
                "resolution": [POST["width"], POST["height"]], "l2": L2_NOTE}
    if w == "batch":
        return {"workload": "64 uneven views of the box (36 tris) and displaced (4,196,562 tris) scenes, "
                            "resolutions 128^2..1920x1080, spp 16/64/256, depth 8/16, RR from 3, extended estimator; "
                            "wavefront form, one graph launch per batch, options and BVH width from the autotuner; "
                            "treelet-optimised BVH",
                "views": 64, "samples_per_step": 4728979456, "l2": L2_NOTE}
    if w == "box":
        return {"workload": "box scene (36 tris) 512x512, 64 spp, 8 segments, RR from 3, extended estimator, " + form,
                "resolution": [512, 512], "spp": 64, "max_bounces": 8, "rr_depth": 3, "l2": L2_NOTE}
    if w == "displaced":
        return {"workload": "displaced icosphere (4,196,562 tris) 1920x1080, 16 spp per step, depth 16, RR from 3, "
                            "extended estimator, " + form, "l2": L2_NOTE}
    if w == "inverse":
        return {"workload": "inverse rendering, box scene with 34 per-triangle albedos + light radiance, 256x256, "
                            "32 spp forward + L2 loss vs a 4096-spp target + 32 spp path-replay backward, depth 8, "
                            "RR from 3", "resolution": [256, 256], "spp_forward": 32, "spp_backward": 32, "l2": L2_NOTE}
    return {"workload": "soup 1,048,576 tris, 16,777,216 closest-hit rays per step, BVH width 8", "l2": L2_NOTE}


# ---------------------------------------------------------------- CPU oracle leg
def cpu_render(scene, camera, st, rows, skybox=None, nthreads=0):
    from oracle import orc

    f = orc.render(scene, camera, st, nthreads=nthreads, rows=rows, skybox=skybox)
    return (rows[1] - rows[0]) * st.width * st.spp, f["render_seconds"]


def cpu_reference_threads(workload):
    """The box frame on the reference's default thread count, a quarter of the
    hardware threads (src/main.cpp:5-6), beside the all-core figure."""
    if workload not in ("box", "batch"):
        return None
    from crender_gb300 import api, scenes

    threads = max(1, (os.cpu_count() or 1) // 4)
    sc = scenes.box_scene()
    n, dt = cpu_render(sc, sc["camera"], api.make_settings(**BOX), (0, 512), nthreads=threads)
    return {"threads": threads, "value": n / dt / 1e6,
            "sample": f"box full frame 512x512x64 ({n} samples, {dt:.1f} s)"}


def cpu_cores(workload):
    """Host threads the CPU leg uses: the post-processing oracle is single-threaded."""
    return 1 if workload == "post" else (os.cpu_count() or 1)


def cpu_leg(workload):
    """Bounded CPU sample of the workload on all host cores (the oracle)."""
    from crender_gb300 import api, scenes
    from oracle import orc

    if workload == "soup":
        v = scenes.soup(1 << 20, 1)
        rays = scenes.soup_rays(1 << 22, 2)
        b = orc.Bvh(v)
        t0 = time.perf_counter()
        b.closest(rays)
        dt = time.perf_counter() - t0
        return (1 << 22) / dt / 1e6, f"4,194,304 of the 16,777,216 primary rays on the soup ({dt:.1f} s)"
    if workload == "post":
        from crender_gb300 import api as capi

        W, H = POST["width"], POST["height"]
        img = post_image(W, H)
        t0 = time.perf_counter()
        orc.post_process(img, post_settings_full(capi))
        dt = time.perf_counter() - t0
        return W * H / dt / 1e6, f"one full 3840x2160 image on one host core ({dt:.1f} s)"
    if workload == "inverse":
        sc = scenes.inverse_box(albedo=np.full((34, 3), 0.5), light_colour=np.full(3, 10 / 17))
        st = api.make_settings(256, 256, 32, 8, 3, 1, 1)
        f = orc.render(sc, sc["camera"], st)
        adj = np.random.default_rng(0).uniform(-1, 1, 256 * 256 * 3).astype(np.float32)
        t0 = time.perf_counter()
        orc.adjoint(sc, sc["camera"], st, adj)
        dt = f["render_seconds"] + time.perf_counter() - t0
        n = 2 * 256 * 256 * 32
        return n / dt / 1e6, f"one full forward + adjoint step of the inverse box, 256x256x32 spp ({n} samples, {dt:.2f} s)"
    n_tot, t_tot, parts = 0, 0.0, []
    if workload in ("box", "batch"):
        sc = scenes.box_scene()
        n, dt = cpu_render(sc, sc["camera"], api.make_settings(**BOX), (0, 512))
        n_tot, t_tot = n_tot + n, t_tot + dt
        parts.append(f"box full frame 512x512x64 ({n} samples, {dt:.1f} s)")
    if workload in ("displaced", "batch"):
        sc = scenes.displaced_scene()
        st = api.make_settings(1920, 1080, 16, 16, 3, 1, 1, 1920 / 1080)
        n, dt = cpu_render(sc, sc["camera"], st, (0, 1080), skybox=sc["skybox"])
        n_tot, t_tot = n_tot + n, t_tot + dt
        parts.append(f"displaced full frame 1920x1080x16 ({n} samples, {dt:.1f} s)")
    return n_tot / t_tot / 1e6, "; ".join(parts)


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    cores = cpu_cores(args.workload)
    vals, sample = [], ""
    for i in range(args.warmup + args.steps):
        v, sample = cpu_leg(args.workload)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    unit = {"soup": "Mrays/s", "post": "Mpixels/s"}.get(args.workload, "Msamples/s")
    cpu = {"value": value, "unit": unit, "cores": cores, "kind": "port", "sample": sample}
    quarter = cpu_reference_threads(args.workload)
    if quarter:
        cpu["reference_default_threads"] = quarter
    print(json.dumps({
        "impl": "reference", "metric": unit, "value": value, "unit": unit, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(args.workload, args.form),
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU oracle: C++ restatement of CRender's estimator with an LBVH + watertight traversal standing in "
                "for Embree 3, which cannot be built here; std::thread over all host cores",
    }))
    return 0


# ---------------------------------------------------------------- GPU helpers
class Timer:
    def __init__(self, torch, stream, flush):
        self.torch, self.stream, self.flush = torch, stream, flush

    def steps(self, fn, steps, warmup):
        """Sum of per-step CUDA-event times (ms) with an L2 flush between steps."""
        for _ in range(warmup):
            fn()
        self.torch.cuda.synchronize()
        evs = [(self.torch.cuda.Event(enable_timing=True), self.torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for e0, e1 in evs:
            self.flush()
            e0.record(self.stream)
            fn()
            e1.record(self.stream)
        self.torch.cuda.synchronize()
        return [e0.elapsed_time(e1) for e0, e1 in evs]


def time_to_rmse(ctx, api, scenes, timer, stream, target=1e-2):
    """Box configuration: spp needed to reach RMSE <= target against an FP64
    16384-spp reference, and the device time of that many spp for each form."""
    sc = scenes.box_scene()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1)
    ref = api.Film(ctx, 512, 512, f64=True)
    ctx.check(api.render_batch([s], [(0, sc["camera"], api.make_settings(512, 512, 16384, 8, 3, 1, 9001))], [ref]))
    r = ref.download(f64=True)["sum64"] / 16384.0
    ref.close()
    film = api.Film(ctx, 512, 512)
    spp, rmse, total = 0, float("inf"), 0
    step = 64
    while rmse > target and total < 16384:
        api.render(s, sc["camera"], api.make_settings(512, 512, step, 8, 3, 1, 1), film, stream)
        total += step
        img = film.download()["sum"].astype(np.float64) / total
        rmse = float(np.sqrt(np.mean((img - r) ** 2)))
        spp = total
    film.close()
    st = api.make_settings(512, 512, spp, 8, 3, 1, 1)
    f = api.Film(ctx, 512, 512)
    s.build(*MEGA_BVH["box"], stream=stream)
    t_mega = timer.steps(lambda: (f.reset(stream), api.render(s, sc["camera"], st, f, stream)), 1, 1)[0]
    tuned, width, _ = api.autotune_batch([s], [(0, sc["camera"], st)], sample_budget=1 << 27, widths=4 | 8, stream=stream,
                                         leaves=LEAVES)
    t_wave = timer.steps(lambda: (f.reset(stream), ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f], tuned, stream))), 1, 1)[0]
    f.close()
    s.close()
    return {"target_rmse": target, "spp": spp, "rmse": rmse, "reference": "FP64 16384-spp box image, independent seed",
            "megakernel_s": t_mega / 1e3, "wavefront_s": t_wave / 1e3,
            "megakernel_bvh": dict(zip(("width", "treelet", "leaf_max"), MEGA_BVH["box"])),
            "wavefront_opts": dict(tuned, width=width), "note": "wavefront options from crg_autotune_batch (untimed)"}


def inverse_workload(ctx, api, scenes, timer, S, args, world, out, torch):
    """Forward / loss / backward step of the inverse-rendering problem, plus FD
    agreement and an Adam run through the public calls."""
    W, SPP = 256, 32
    true_sc = scenes.inverse_box()
    init = scenes.inverse_box(albedo=np.full((34, 3), 0.5), light_colour=np.full(3, 10 / 17))
    scene = api.Scene(ctx, init["verts"], init["mat_idx"], init["mats"]).build(8, 1)
    cam = init["camera"]
    nmat, npx = len(init["mats"]), W * W * 3
    # target: 4096 spp of the true parameters, FP64 film
    api.set_materials(scene, true_sc["mats"])
    tf = api.Film(ctx, W, W, f64=True)
    api.render(scene, cam, api.make_settings(W, W, 4096, 8, 3, 1, 4242), tf, S)
    target = (tf.download(f64=True)["sum64"] / 4096).astype(np.float32)
    tf.close()
    api.set_materials(scene, init["mats"])
    tb = api.DeviceBuffer.from_array(ctx, target)
    ab, lb = api.DeviceBuffer(ctx, npx * 4), api.DeviceBuffer(ctx, 8)
    gc, ge = api.DeviceBuffer(ctx, nmat * 24), api.DeviceBuffer(ctx, nmat * 8)
    film = api.Film(ctx, W, W)
    fwd = api.make_settings(W, W, SPP, 8, 3, 1, 1)
    bwd = api.make_settings(W, W, SPP, 8, 3, 1, 2)

    def forward():
        film.reset(S)
        api.render(scene, cam, fwd, film, S)
        api.loss_l2(film, tb, ab, lb, S)

    def backward():
        api.backward(scene, cam, bwd, ab, gc, ge, S)

    def step():
        forward()
        backward()

    # traversal work of the backward pass (the forward with the backward's random numbers traces the same paths)
    scene.set_counting(True)
    film.reset(S)
    api.render(scene, cam, bwd, film, S)
    torch.cuda.synchronize()
    work = scene.stats()
    scene.set_counting(False)
    units = 2 * W * W * SPP
    algo = 2 * (work["nodes_visited"] * scene.info()["node_bytes"] + work["tris_tested"] * 48) + W * W * 12 * 4
    with ClockSampler(env_rank()[2]) as clk:
        ms = timer.steps(step, args.steps, args.warmup)
    f_ms = timer.steps(forward, 3, 1)
    b_ms = timer.steps(backward, 3, 1)
    out["work"] = {**work, "note": "counted on the forward with the backward's random numbers (same paths)"}
    out["forward_ms"] = statistics.median(f_ms)
    out["backward_ms"] = statistics.median(b_ms)
    out["backward_over_forward"] = out["backward_ms"] / out["forward_ms"]

    # central differences with common random numbers (roulette off) against the adjoint
    f64film = api.Film(ctx, W, W, f64=True)
    st0 = api.make_settings(W, W, SPP, 8, 0, 1, 7)
    f64film.reset(S)
    api.render(scene, cam, st0, f64film, S)
    img = f64film.download(f64=True)["sum64"] / SPP
    adj = (2.0 * (img - target) / npx).astype(np.float32)
    ab.upload(adj)
    gc.upload(np.zeros(nmat * 3))
    ge.upload(np.zeros(nmat))
    api.backward(scene, cam, st0, ab, gc, ge, S)
    g = gc.download(np.zeros(nmat * 3)).reshape(nmat, 3)
    h, rel = 1e-3, []
    for m, c in [(0, 0), (6, 1), (14, 2), (26, 0), (34, 1)]:
        vals = []
        for sgn in (1, -1):
            mats = init["mats"].copy()
            mats[m]["colour"][c] += sgn * h
            api.set_materials(scene, mats)
            f64film.reset(S)
            api.render(scene, cam, st0, f64film, S)
            vals.append(float(np.dot(adj.astype(np.float64), f64film.download(f64=True)["sum64"] / SPP)))
        fd = (vals[0] - vals[1]) / (2 * h)
        rel.append(abs(g[m, c] - fd) / max(abs(fd), 1e-30))
    api.set_materials(scene, init["mats"])
    f64film.close()
    out["fd_check"] = {"params": 5, "h": h, "max_rel_err": max(rel), "spp": SPP, "resolution": [W, W],
                       "rr": "off", "random_numbers": "common (same seed for +h, -h and the adjoint)"}

    # e2e: Adam through the public calls, host parameters, per-step uploads and gradient downloads
    theta = np.concatenate([np.full(102, 0.5), np.full(3, 10 / 17)])
    hi = np.concatenate([np.ones(102), np.full(3, 4.0)])
    m1, m2 = np.zeros_like(theta), np.zeros_like(theta)
    zc, ze, lh = np.zeros(nmat * 3), np.zeros(nmat), np.zeros(1)
    losses = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(200):
        mats = scenes.inverse_box(albedo=theta[:102].reshape(34, 3), light_colour=theta[102:])["mats"]
        api.set_materials(scene, mats)
        fwd.seed, bwd.seed = 1000 + 2 * it, 1001 + 2 * it
        gc.upload(zc, S)
        ge.upload(ze, S)
        forward()
        backward()
        lb.download(lh, S)
        grad = gc.download(zc.copy(), S)[:105]  # 34 albedos (RGB) then the light colour
        if it == 0:
            g_first = np.abs(grad[:102]).copy()
        losses.append(float(lh[0]))
        m1 = 0.9 * m1 + 0.1 * grad
        m2 = 0.999 * m2 + 0.001 * grad * grad
        theta = np.clip(theta - 0.02 * (m1 / (1 - 0.9 ** (it + 1))) / (np.sqrt(m2 / (1 - 0.999 ** (it + 1))) + 1e-12),
                        1e-3, hi)
    torch.cuda.synchronize()
    adam_s = time.perf_counter() - t0
    truth = true_sc["true_albedo"].ravel()
    out["adam"] = {"steps": 200, "lr": 0.02, "seconds": adam_s, "loss_first": losses[0],
                   "loss_last10_mean": float(np.mean(losses[-10:])),
                   "albedo_mae_first": float(np.abs(0.5 - truth).mean()),
                   "albedo_mae_last": float(np.abs(theta[:102] - truth).mean()),
                   "light_radiance_last": (17 * theta[102:]).tolist(), "light_radiance_true": 17.0}
    # which albedos the image constrains: the first step's gradient magnitude per parameter against
    # the final error (a parameter whose gradient is tiny barely moves the loss, so Adam's steps on
    # it follow noise)
    err = np.abs(theta[:102] - truth)
    weak = g_first < 1e-2 * g_first.max()
    order = np.argsort(g_first)
    third = len(order) // 3
    out["adam"]["constraint"] = {
        "how": "first-step |dL/d albedo| per parameter (34 triangles x RGB) against the final |albedo error|",
        "weak_params": int(weak.sum()), "weak_threshold": "below 1e-2 of the largest gradient",
        "mae_weak": float(err[weak].mean()) if weak.any() else None,
        "mae_rest": float(err[~weak].mean()) if (~weak).any() else None,
        "mae_by_gradient_third": [float(err[order[:third]].mean()), float(err[order[third:2 * third]].mean()),
                                  float(err[order[2 * third:]].mean())]}
    h2d = nmat * 48 + nmat * 24 + nmat * 8
    out["e2e"] = {"value": units * world / (adam_s / 200) / 1e6, "unit": "Msamples/s", "h2d_bytes_per_step": h2d,
                  "d2h_bytes_per_step": 8 + nmat * 24, "ms_per_step": adam_s / 200 * 1e3,
                  "path": "crg_scene_set_materials (host table) + crg_render + crg_film_loss_l2 + crg_backward + "
                          "loss and gradient downloads + host Adam update, 200 iterations"}
    for b in (tb, ab, lb, gc, ge):
        b.free()
    film.close()
    scene.close()
    return units, algo, "k_render + k_loss_l2 + k_adjoint (one forward/backward step)", 3 * args.steps, clk, ms


def max_over_ranks(seconds, world, device):
    """The slowest rank's timed-region length (replicas: every rank renders its own
    copy of the workload), then a barrier so no rank leaves early."""
    if world <= 1:
        return seconds
    import torch
    import torch.distributed as dist

    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def weak_scaling_value(units, steps, world, seconds):
    """Whole-job throughput in millions of units per second: every rank processed
    `units` per step."""
    return units * steps * world / seconds / 1e6


def wavefront_overrides(args):
    """Wavefront options given on the command line (host-driven loop, path pool size)."""
    o = {}
    if args.host_loop:
        o["host_loop"] = 1
    if args.path_pool:
        o["path_pool"] = args.path_pool
    return o


# ---------------------------------------------------------------- GPU leg
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="crg", choices=["crg", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "box", "displaced", "soup", "inverse", "post"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-rmse", action="store_true", help="skip the time-to-RMSE leg")
    ap.add_argument("--form", default="megakernel", choices=["megakernel", "wavefront"],
                    help="renderer for the box / displaced workloads")
    ap.add_argument("--host-loop", action="store_true",
                    help="wavefront: drive the loop from the host (profilers cannot see kernels inside "
                         "graphs with conditional nodes)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batch: use the autotuner's usual pick instead of running it (profiler runs)")
    ap.add_argument("--spp-div", type=int, default=1,
                    help="batch: divide every view's spp by this (a smaller copy of the batch for profiler captures; "
                         "the JSON line then names the reduced samples per step)")
    ap.add_argument("--path-pool", type=int, default=0,
                    help="wavefront: paths in flight (0 = the autotuned or default pool); smaller pools keep "
                         "profiler captures within a few GB of device memory")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from crender_gb300 import api, scenes

    ctx = api.Context(local)
    stream = torch.cuda.current_stream()
    S = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    timer = Timer(torch, stream, lambda: flush.fill_(rank & 0xFF))
    peak, peak_kind = measured_peaks()
    out = {}
    unit = {"soup": "Mrays/s", "post": "Mpixels/s"}.get(args.workload, "Msamples/s")

    if args.workload == "batch":
        box, disp = scenes.box_scene(), scenes.displaced_scene()
        sb = api.Scene(ctx, box["verts"], box["mat_idx"], box["mats"]).build(8, 1)
        sd = api.Scene(ctx, disp["verts"], disp["mat_idx"], disp["mats"]).build(8, 1)
        sd.set_skybox(disp["skybox"])
        vdefs = scenes.batch_views()
        div = max(1, args.spp_div)
        views = [(si, cam, api.make_settings(v["width"], v["height"], max(1, v["spp"] // div), v["max_bounces"], 3, 1,
                                             1 + i, v["width"] / v["height"])) for i, (si, cam, v) in enumerate(vdefs)]
        films = [api.Film(ctx, st.width, st.height) for _, _, st in views]
        units = sum(st.width * st.height * st.spp for _, _, st in views)
        out["scene_samples"] = {name: sum(st.width * st.height * st.spp for si, _, st in views if si == k)
                                for k, name in enumerate(("box", "displaced"))}

        # autotuner (untimed): BVH width, stage fusion, refill, fetch, block size, path pool
        t0 = time.perf_counter()
        if args.no_autotune:
            # options the autotuner picks for this batch on a GB300 (fixed, so profiler runs launch no tuning graphs)
            tuned, tuned_width = dict(path_pool=1 << 27, chunk_samples=1 << 27, block_size=256, fetch=64,
                                      max_iterations=0, count_work=0, host_loop=0, fuse=1, refill=16), 8
            out["autotune"] = {"skipped": True, "width": tuned_width, "opts": tuned}
        else:
            tuned, tuned_width, trials = api.autotune_batch([sb, sd], views, sample_budget=1 << 28, widths=2 | 4 | 8,
                                                            stream=S, leaves=LEAVES)
            out["autotune"] = {"seconds": time.perf_counter() - t0, "width": tuned_width, "opts": tuned,
                               "leaf_max": {"box": sb.info()["leaf_max"], "displaced": sd.info()["leaf_max"]},
                               "trials": len(trials), "trial_batch_samples": 1 << 28,
                               "best_trial_msamples_per_s": max(t["msamples_per_s"] for t in trials)}
        tuned = dict(tuned, **wavefront_overrides(args))

        def wave():
            for f in films:
                f.reset(S)
            ctx.check(api.render_batch([sb, sd], views, films, tuned, S))

        def mega():
            for (si, cam, st), f in zip(views, films):
                f.reset(S)
                api.render((sb, sd)[si], cam, st, f, S)

        # instrumented wavefront pass (untimed, host-driven loop): traversal work of each traversal stage
        for f in films:
            f.reset(S)
        ctx.check(api.render_batch([sb, sd], views, films, dict(tuned, count_work=1, host_loop=2), S))
        torch.cuda.synchronize()
        work = api.batch_stats(ctx)
        sh_work = api.stage_times(ctx)
        rays = work["segments"] + work["shadow_rays"]
        nb = sd.info()["node_bytes"]
        algo = rays * 48 + work["nodes_visited"] * nb + work["tris_tested"] * 48 + units * 12
        with ClockSampler(local) as clk:
            ms = timer.steps(wave, args.steps, args.warmup)
        # one more frame through the host-driven loop with CUDA events around every stage (untimed above):
        # the device time of each kernel stage, for the dominant kernel's roofline and the frame's time shares
        for f in films:
            f.reset(S)
        ctx.check(api.render_batch([sb, sd], views, films, dict(tuned, host_loop=2), S))
        torch.cuda.synchronize()
        out["stages"] = stage_roofline(tuned, work, sh_work, api.stage_times(ctx), nb, peak)
        # per view size: the wavefront form against the megakernel on the views of each resolution
        sizes = sorted({(st.width, st.height) for _, _, st in views}, key=lambda wh: wh[0] * wh[1])
        groups = {wh: [i for i, (_, _, st) in enumerate(views) if (st.width, st.height) == wh] for wh in sizes}
        by_size = {}
        for wh, idx in groups.items():
            sv, sf = [views[i] for i in idx], [films[i] for i in idx]

            def wave_part(sv=sv, sf=sf):
                for f in sf:
                    f.reset(S)
                ctx.check(api.render_batch([sb, sd], sv, sf, tuned, S))

            t = timer.steps(wave_part, 1, 1)[0]
            n = sum(st.width * st.height * st.spp for _, _, st in sv)
            by_size[f"{wh[0]}x{wh[1]}"] = {"views": len(idx), "samples": n, "wavefront_msamples_per_s": n / t / 1e3}
        wave_leaf = (sb.info()["leaf_max"], sd.info()["leaf_max"])
        sb.build(*MEGA_BVH["box"], stream=S)  # the megakernel runs on its own best BVHs
        sd.build(*MEGA_BVH["displaced"], stream=S)
        for wh, idx in groups.items():
            sv, sf = [views[i] for i in idx], [films[i] for i in idx]

            def mega_part(sv=sv, sf=sf):
                for (si, cam, st), f in zip(sv, sf):
                    f.reset(S)
                    api.render((sb, sd)[si], cam, st, f, S)

            t = timer.steps(mega_part, 1, 1)[0]
            e = by_size[f"{wh[0]}x{wh[1]}"]
            e["megakernel_msamples_per_s"] = e["samples"] / t / 1e3
            e["wavefront_over_megakernel"] = e["wavefront_msamples_per_s"] / e["megakernel_msamples_per_s"]
        out["by_view_size"] = by_size
        mega_steps, mega_warm = args.steps, args.warmup
        mega_ms = timer.steps(mega, mega_steps, mega_warm)
        out["megakernel"] = {"value": units / (sum(mega_ms) / len(mega_ms) / 1e3) / 1e6, "unit": unit,
                             "ms_per_step": sum(mega_ms) / len(mega_ms), "ms_min": min(mega_ms), "ms_max": max(mega_ms),
                             "steps": mega_steps, "warmup": mega_warm,
                             "bvh": {k: dict(zip(("width", "treelet", "leaf_max"), v)) for k, v in MEGA_BVH.items()},
                             "how": "same 64 views, one crg_render call per view (the drop-in), on the BVH options "
                                    "fastest for the megakernel in a sweep of width x leaf size; the wavefront arm's "
                                    "warm-up and timed steps, L2 flushed between steps"}
        out["work"] = {**work, "mrays_per_step": rays / 1e6, "shadow_nodes_visited": sh_work["shadow_nodes"],
                       "shadow_tris_tested": sh_work["shadow_tris"]}
        kernel = "wavefront frame: one graph launch (k_wf_extend / k_wf_shade / k_wf_shadow / control / resolve)"
        launches = None  # counted below from the iteration count

        # e2e: both scenes from pinned host memory, build, batch render, all films back to pinned memory
        pins = {}
        for name, sc in (("box", box), ("disp", disp)):
            pins[name] = [api.PinnedArray(ctx, sc[k].shape, sc[k].dtype) for k in ("verts", "mat_idx", "mats")]
            for p, k in zip(pins[name], ("verts", "mat_idx", "mats")):
                p.array[...] = sc[k]
        outs = [api.PinnedArray(ctx, (st.width * st.height * 3,), np.float32) for _, _, st in views]
        h2d = sum(p.array.nbytes for v in pins.values() for p in v) + 16
        d2h = sum(o.array.nbytes for o in outs)

        def e2e_step():
            a = api.Scene(ctx, *[p.array for p in pins["box"]]).build(tuned_width, 1, wave_leaf[0], stream=S)
            b = api.Scene(ctx, *[p.array for p in pins["disp"]]).build(tuned_width, 1, wave_leaf[1], stream=S)
            b.set_skybox(disp["skybox"])
            for f in films:
                f.reset(S)
            ctx.check(api.render_batch([a, b], views, films, tuned, S))
            for f, o in zip(films, outs):  # the 64 copies enqueued, one wait
                ctx.check(ctx.lib.crg_film_download_async(f.h, o.ptr, None, None, None, None, None, S))
            ctx.check(ctx.lib.crg_stream_sync(ctx.h, S))
            a.close()
            b.close()

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / 2
        out["e2e"] = {"value": units * world / e2e_s / 1e6, "unit": unit, "h2d_bytes_per_step": int(h2d),
                      "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                      "path": "crg_scene_create x2 (pinned host geometry) + crg_scene_build x2 + crg_render_batch + "
                              "64 x crg_film_download_async (pinned) + one crg_stream_sync"}
        if not args.no_rmse:
            out["time_to_rmse"] = time_to_rmse(ctx, api, scenes, timer, S)
    elif args.workload in ("box", "displaced"):
        if args.workload == "box":
            sc = scenes.box_scene()
            st = api.make_settings(**BOX)
        else:
            sc = scenes.displaced_scene()
            st = api.make_settings(1920, 1080, 16, 16, 3, 1, 1, 1920 / 1080)
        # the megakernel on its own best BVH; the wavefront form on width 8 with the leaf size its tuner
        # picks for each scene (box 3, displaced 1)
        bvh = MEGA_BVH[args.workload] if args.form == "megakernel" else (8, 1, 3 if args.workload == "box" else 1)
        scene = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(*bvh)
        out["bvh"] = dict(zip(("width", "treelet", "leaf_max"), bvh))
        if "skybox" in sc:
            scene.set_skybox(sc["skybox"])
        film = api.Film(ctx, st.width, st.height)
        units = st.width * st.height * st.spp

        if args.form == "megakernel":
            def step():
                film.reset(S)
                api.render(scene, sc["camera"], st, film, S)

            scene.set_counting(True)
            step()
            torch.cuda.synchronize()
            work = scene.stats()
            scene.set_counting(False)
            kernel = "k_render (megakernel)"
            launches = args.steps
        else:
            wopts = wavefront_overrides(args) or None

            def step():
                film.reset(S)
                ctx.check(api.render_batch([scene], [(0, sc["camera"], st)], [film], wopts, S))

            film.reset(S)
            ctx.check(api.render_batch([scene], [(0, sc["camera"], st)], [film], dict(wopts or {}, count_work=1), S))
            torch.cuda.synchronize()
            work = api.batch_stats(ctx)
            kernel = "wavefront frame: one graph launch"
            launches = args.steps * (3 + 7 * int(work["iterations"]))
        rays = work["segments"] + work["shadow_rays"]
        algo = work["nodes_visited"] * scene.info()["node_bytes"] + work["tris_tested"] * 48 + units * 12
        out["work"] = {**work, "mrays_per_step": rays / 1e6}
        out["form"] = args.form
        with ClockSampler(local) as clk:
            ms = timer.steps(step, args.steps, args.warmup)
        pv = api.PinnedArray(ctx, sc["verts"].shape, np.float32)
        pm = api.PinnedArray(ctx, sc["mat_idx"].shape, np.uint32)
        pmat = api.PinnedArray(ctx, sc["mats"].shape, sc["mats"].dtype)
        pout = api.PinnedArray(ctx, (st.width * st.height * 3,), np.float32)
        pv.array[...], pm.array[...], pmat.array[...] = sc["verts"], sc["mat_idx"], sc["mats"]

        def e2e_step():
            s2 = api.Scene(ctx, pv.array, pm.array, pmat.array).build(*bvh, stream=S)
            if "skybox" in sc:
                s2.set_skybox(sc["skybox"])
            film.reset(S)
            if args.form == "megakernel":
                api.render(s2, sc["camera"], st, film, S)
            else:
                ctx.check(api.render_batch([s2], [(0, sc["camera"], st)], [film], wopts, S))
            ctx.check(ctx.lib.crg_film_download(film.h, pout.ptr, None, None, None, None, None, S))
            s2.close()

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.steps
        out["e2e"] = {"value": units * world / e2e_s / 1e6, "unit": unit,
                      "h2d_bytes_per_step": int(pv.array.nbytes + pm.array.nbytes + pmat.array.nbytes),
                      "d2h_bytes_per_step": int(pout.array.nbytes), "ms_per_step": e2e_s * 1e3,
                      "path": "crg_scene_create (pinned host geometry) + crg_scene_build + "
                              + ("crg_render" if args.form == "megakernel" else "crg_render_batch") + " + crg_film_download"}
        if args.workload == "box" and not args.no_rmse:
            out["time_to_rmse"] = time_to_rmse(ctx, api, scenes, timer, S)
    elif args.workload == "inverse":
        units, algo, kernel, launches, clk, ms = inverse_workload(ctx, api, scenes, timer, S, args, world, out, torch)
    elif args.workload == "post":
        unit = "Mpixels/s"
        W, H = POST["width"], POST["height"]
        img = post_image(W, H)
        src = api.DeviceBuffer.from_array(ctx, img)
        dst = api.DeviceBuffer(ctx, img.nbytes)
        ps = post_settings_full(api)
        units = W * H
        # per pixel: pass 0 reads the source and writes 16 B, passes 1-9 read and write 16 B each,
        # the composite reads source + bloom and writes the output
        algo = units * (10 * 32 + 48)

        def step():
            api.post_process(ctx, src, dst, W, H, ps, S)

        with ClockSampler(local) as clk:
            ms = timer.steps(step, args.steps, args.warmup)
        kernel = "k_blur_h / k_blur_v x 10 + k_post_final (one crg_post_process call)"
        launches = 11 * args.steps
        pin_in = api.PinnedArray(ctx, img.shape, np.float32)
        pin_out = api.PinnedArray(ctx, img.shape, np.float32)
        pin_in.array[...] = img

        def e2e_step():
            ctx.check(ctx.lib.crg_memcpy_h2d(ctx.h, src.ptr, pin_in.ptr, img.nbytes, S))
            api.post_process(ctx, src, dst, W, H, ps, S)
            ctx.check(ctx.lib.crg_memcpy_d2h(ctx.h, pin_out.ptr, dst.ptr, img.nbytes, S))
            ctx.check(ctx.lib.crg_stream_sync(ctx.h, S))

        e2e_step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        e2e_s = (time.perf_counter() - t0) / args.steps
        out["e2e"] = {"value": units * world / e2e_s / 1e6, "unit": unit, "h2d_bytes_per_step": int(img.nbytes),
                      "d2h_bytes_per_step": int(img.nbytes), "ms_per_step": e2e_s * 1e3,
                      "path": "crg_memcpy_h2d (pinned image) + crg_post_process + crg_memcpy_d2h (pinned)"}
    else:
        v = scenes.soup(1 << 20, 1)
        scene = api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}])).build()
        n = 1 << 24
        rays_h = scenes.soup_rays(n, 2)
        rb = api.DeviceBuffer.from_array(ctx, rays_h)
        hb = api.DeviceBuffer(ctx, 16 * n)
        units = n
        lib = ctx.lib

        def step():
            ctx.check(lib.crg_intersect_closest(scene.h, rb.ptr, hb.ptr, n, S))

        nb, tb = api.DeviceBuffer(ctx, 4 * n), api.DeviceBuffer(ctx, 4 * n)
        ctx.check(lib.crg_intersect_closest_counted(scene.h, rb.ptr, hb.ptr, nb.ptr, tb.ptr, n, S))
        nodes = int(nb.download(np.zeros(n, np.uint32)).astype(np.int64).sum())
        tris = int(tb.download(np.zeros(n, np.uint32)).astype(np.int64).sum())
        algo = n * 48 + nodes * scene.info()["node_bytes"] + tris * 48
        out["work"] = {"nodes_visited": nodes, "tris_tested": tris}
        with ClockSampler(local) as clk:
            ms = timer.steps(step, args.steps, args.warmup)
        kernel = "k_intersect<8> (closest hit)"
        launches = args.steps
        # any-hit leg: 16,777,216 shadow rays of the same generator (separate seed, tmax ~ U[0.1, 1])
        sb = api.DeviceBuffer.from_array(ctx, scenes.soup_rays(n, 3, shadow=True))
        ob = api.DeviceBuffer(ctx, 4 * n)
        ms_any = timer.steps(lambda: ctx.check(lib.crg_intersect_any(scene.h, sb.ptr, ob.ptr, n, S)),
                             args.steps, args.warmup)
        occluded = int(ob.download(np.zeros(n, np.uint32)).astype(bool).sum())
        out["any_hit"] = {"value": n / (sum(ms_any) / len(ms_any) / 1e3) / 1e6, "unit": "Mrays/s",
                          "ms_per_step": sum(ms_any) / len(ms_any), "rays": n, "occluded_fraction": occluded / n,
                          "kernel": "k_intersect_dyn<8> (any hit, per-lane refill)"}
        # the warp-cooperative scheme on the same rays (8 lanes per ray, nodes staged in shared memory)
        ms_wc = timer.steps(lambda: ctx.check(lib.crg_intersect_closest_with(scene.h, rb.ptr, hb.ptr, n,
                                                                             api.TRAVERSAL_WARP, S)),
                            args.steps, args.warmup)
        ms_wa = timer.steps(lambda: ctx.check(lib.crg_intersect_any_with(scene.h, sb.ptr, ob.ptr, n,
                                                                         api.TRAVERSAL_WARP, S)),
                            args.steps, args.warmup)
        out["warp_traversal"] = {
            "closest_mrays_per_s": n / (sum(ms_wc) / len(ms_wc) / 1e3) / 1e6,
            "any_mrays_per_s": n / (sum(ms_wa) / len(ms_wa) / 1e3) / 1e6, "rays": n,
            "kernel": "k_intersect_warp<8> (crg_intersect_*_with, CRG_TRAVERSAL_WARP)"}
        sb.free()
        ob.free()
        pr = api.PinnedArray(ctx, rays_h.shape, rays_h.dtype)
        pr.array[...] = rays_h
        ph = api.PinnedArray(ctx, (n * 16,), np.uint8)

        def e2e_step():
            ctx.check(lib.crg_memcpy_h2d(ctx.h, rb.ptr, pr.ptr, pr.array.nbytes, S))
            ctx.check(lib.crg_intersect_closest(scene.h, rb.ptr, hb.ptr, n, S))
            ctx.check(lib.crg_memcpy_d2h(ctx.h, ph.ptr, hb.ptr, n * 16, S))
            ctx.check(lib.crg_stream_sync(ctx.h, S))

        e2e_step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        e2e_s = (time.perf_counter() - t0) / args.steps
        out["e2e"] = {"value": units * world / e2e_s / 1e6, "unit": unit, "h2d_bytes_per_step": int(pr.array.nbytes),
                      "d2h_bytes_per_step": int(n * 16), "ms_per_step": e2e_s * 1e3,
                      "path": "crg_memcpy_h2d (pinned rays) + crg_intersect_closest + crg_memcpy_d2h (pinned hits)"}

    total_s = max_over_ranks(sum(ms) / 1e3, world, "cuda")
    value = weak_scaling_value(units, args.steps, world, total_s)
    achieved = algo / (total_s / args.steps) / 1e9
    if launches is None:
        # per frame: 3 prologue kernels + per device-loop iteration: the bounce kernels (3 split, 2 with the shadow
        # test in shade, 1 fused) + control, resolve, generate, generated
        fuse = out.get("autotune", {}).get("opts", {}).get("fuse", 1) or 1
        launches = args.steps * (3 + (4 + (3, 2, 1)[fuse - 1]) * int(out["work"]["iterations"]))
    traffic, traffic_src = traffic_estimate(args.workload, out, units)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "traffic_source": traffic_src, "kernel": kernel, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": int(algo)}
    if args.workload == "batch" and out.get("stages", {}).get("dominant"):
        # the dominant kernel: the largest traversal stage of the frame, timed by its own CUDA events
        st = out["stages"]
        d = st["traversal"][st["dominant"]]
        frame = dict(roofline, kernel="whole frame (all stages): " + kernel)
        roofline = {"bound": "hbm", "achieved": d["achieved_gbs"], "peak": peak, "unit": "GB/s",
                    "frac": d["frac"], "traffic": traffic_dominant(out, st["dominant"]),
                    "traffic_source": "DRAM bytes per ray of the same kernel in an ncu capture of a displaced-scene "
                                      "iteration, times the frame's rays of that stage (an upper estimate: the box "
                                      "scene's rays find its BVH in L1/L2)",
                    "kernel": d["kernel"] + f" ({st['dominant']} stage, {st['share'][st['dominant']]:.2f} of the frame)",
                    "peak_kind": peak_kind, "algorithmic_bytes_per_frame": d["algorithmic_bytes"],
                    "stage_ms_per_frame": d["ms"], "l2_hit_rate": L2_HIT.get(st["dominant"]),
                    "l2_hit_rate_source": "ncu lts__t_sector_hit_rate of the same kernel on the displaced scene "
                                          "(profiles/wavefront_displaced_iteration_full.md)",
                    "stage_share": st["share"], "frame": frame}
    elif args.workload == "soup":
        roofline["l2_hit_rate"] = L2_HIT["soup_closest"]
        roofline["l2_hit_rate_source"] = "ncu capture of the same launch (profiles/k_intersect_soup_full.md)"
    config = workload_config(args.workload, args.form)
    if args.workload == "batch":
        config["samples_per_step"] = units
        if args.spp_div > 1:
            config["spp_div"] = args.spp_div
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cv, sample = cpu_leg(args.workload)
        cpu = {"value": cv, "unit": unit, "cores": cpu_cores(args.workload), "kind": "port", "sample": sample}
        quarter = cpu_reference_threads(args.workload)
        if quarter:
            cpu["reference_default_threads"] = quarter
    if rank == 0:
        line = {
            "metric": unit, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config,
            "roofline": roofline,
            "cpu_baseline": cpu, "clocks": clk.summary(), "gpu_launches": launches, **out,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
