#!/usr/bin/env python3
"""Benchmark of the render hot path through the C ABI (libcrg.so).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl crg|reference]
                    [--workload box|soup]

Workloads (seeded synthetic inputs; no external data):
  box   the 36-triangle box scene, 512x512, 64 spp, 8 segments, Russian
        roulette from segment 3, extended estimator (NEE + MIS), one frame
        per step rendered by the one-thread-per-pixel megakernel.
        Metric: Msamples/s (pixel samples).
  soup  1,048,576-triangle soup, 16,777,216 closest-hit rays per step.
        Metric: Mrays/s.

`value` is device-timed (CUDA events on the launching stream, inputs resident,
L2 flushed by a 256 MiB write between steps, outside the events).  `e2e` times
the same step through the public C ABI from pinned host buffers: scene upload,
BVH build, render, film download.  --impl reference times the CPU oracle (the
C++ restatement of the reference integrator, all host cores) on a bounded
sample of the same workload.  Multi-GPU runs are independent replicas (weak
scaling, no collective on the data path).
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
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
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


# ---------------------------------------------------------------- CPU oracle leg
def cpu_box(sample_rows: int, nthreads: int = 0):
    """Times the oracle (C++ restatement of the reference estimator) on rows
    [0, sample_rows) of the box frame.  Returns (Msamples/s, seconds, samples)."""
    from crender_gb300 import api, scenes
    from oracle import orc

    sc = scenes.box_scene()
    st = api.make_settings(**BOX)
    t0 = time.perf_counter()
    orc.render(sc, sc["camera"], st, nthreads=nthreads, rows=(0, sample_rows))
    dt = time.perf_counter() - t0
    n = sample_rows * BOX["width"] * BOX["spp"]
    return n / dt / 1e6, dt, n


def cpu_soup(nrays: int, nthreads: int = 0):
    from crender_gb300 import scenes
    from oracle import orc

    v = scenes.soup(1 << 20, 1)
    rays = scenes.soup_rays(nrays, 2)
    b = orc.Bvh(v)
    t0 = time.perf_counter()
    b.closest(rays, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return nrays / dt / 1e6, dt, nrays


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    cores = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        if args.workload == "box":
            v, dt, n = cpu_box(64)
            sample = "rows 0-63 of the 512x512 64-spp box frame (2,097,152 samples)"
        else:
            v, dt, n = cpu_soup(1 << 18)
            sample = "262,144 of the 16,777,216 primary rays on the 1,048,576-triangle soup"
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    unit = "Msamples/s" if args.workload == "box" else "Mrays/s"
    line = {
        "impl": "reference",
        "metric": unit,
        "value": value,
        "unit": unit,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(args.workload),
        "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU oracle (C++ restatement of CRender's estimator and an LBVH + watertight traversal "
                "standing in for Embree 3, which cannot be built here); std::thread over all host cores",
    }
    print(json.dumps(line))
    return 0


def workload_config(w):
    if w == "box":
        return {"workload": "box scene (36 tris) 512x512, 64 spp, 8 segments, RR from segment 3, extended estimator, "
                            "megakernel, BVH width 8",
                "resolution": [512, 512], "spp": 64, "max_bounces": 8, "rr_depth": 3,
                "l2": "flushed between steps (256 MiB write, outside the timed events)"}
    return {"workload": "soup 1,048,576 tris, 16,777,216 closest-hit rays per step, BVH width 8",
            "l2": "flushed between steps (256 MiB write, outside the timed events)"}


# ---------------------------------------------------------------- GPU leg
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="crg", choices=["crg", "reference"])
    ap.add_argument("--workload", default="box", choices=["box", "soup"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
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
    sh = C_stream = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def flush_l2():
        flush.fill_(rank & 0xFF)

    peak, peak_kind = measured_peaks()
    extra = {}
    if args.workload == "box":
        sc = scenes.box_scene()
        scene = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build()
        st = api.make_settings(**BOX)
        film = api.Film(ctx, 512, 512)
        units_per_step = 512 * 512 * BOX["spp"]
        unit = "Msamples/s"

        def step():
            film.reset(C_stream)
            api.render(scene, sc["camera"], st, film, C_stream)

        # instrumented run (untimed): traversal work for the algorithmic-byte count
        scene.set_counting(True)
        film.reset(C_stream)
        api.render(scene, sc["camera"], st, film, C_stream)
        torch.cuda.synchronize()
        stats = scene.stats()
        scene.set_counting(False)
        node_bytes = scene.info()["node_bytes"]
        rays = stats["segments"] + stats["shadow_rays"]
        # layout-counted bytes: node loads + triangle loads (48 B) + 12 B film RGB per sample
        algo_bytes = stats["nodes_visited"] * node_bytes + stats["tris_tested"] * 48 + units_per_step * 12
        extra["work"] = {"segments": stats["segments"], "shadow_rays": stats["shadow_rays"],
                         "nodes_visited": stats["nodes_visited"], "tris_tested": stats["tris_tested"],
                         "mrays_per_frame": rays / 1e6}
        launches_per_step = 1
        kernel = "k_render (megakernel)"
    else:
        v = scenes.soup(1 << 20, 1)
        scene = api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}])).build()
        rays_h = scenes.soup_rays(1 << 24, 2)
        rb = api.DeviceBuffer.from_array(ctx, rays_h)
        hb = api.DeviceBuffer(ctx, 16 << 24)
        units_per_step = 1 << 24
        unit = "Mrays/s"
        lib = ctx.lib

        def step():
            ctx.check(lib.crg_intersect_closest(scene.h, rb.ptr, hb.ptr, units_per_step, C_stream))

        nb = api.DeviceBuffer(ctx, 4 << 24)
        tb = api.DeviceBuffer(ctx, 4 << 24)
        ctx.check(lib.crg_intersect_closest_counted(scene.h, rb.ptr, hb.ptr, nb.ptr, tb.ptr, units_per_step, C_stream))
        nodes = nb.download(np.zeros(1 << 24, np.uint32)).astype(np.int64).sum()
        tris = tb.download(np.zeros(1 << 24, np.uint32)).astype(np.int64).sum()
        node_bytes = scene.info()["node_bytes"]
        algo_bytes = units_per_step * (32 + 16) + nodes * node_bytes + tris * 48
        extra["work"] = {"nodes_visited": int(nodes), "tris_tested": int(tris)}
        launches_per_step = 1
        kernel = "k_intersect<8> (closest hit)"

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for e0, e1 in evs:
            flush_l2()
            e0.record(stream)
            step()
            e1.record(stream)
        torch.cuda.synchronize()
    ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    total_s = sum(ms) / 1e3
    if world > 1:
        t = torch.tensor([total_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
        torch.distributed.barrier()
    value = units_per_step * args.steps * world / total_s / 1e6
    mean_launch_s = total_s / args.steps
    achieved = algo_bytes / mean_launch_s / 1e9

    # ---- end to end through the C ABI from pinned host buffers
    e2e = None
    if args.workload == "box":
        pv = api.PinnedArray(ctx, sc["verts"].shape, np.float32)
        pm = api.PinnedArray(ctx, sc["mat_idx"].shape, np.uint32)
        pmat = api.PinnedArray(ctx, sc["mats"].shape, sc["mats"].dtype)
        pout = api.PinnedArray(ctx, (512 * 512 * 3,), np.float32)
        pv.array[...] = sc["verts"]
        pm.array[...] = sc["mat_idx"]
        pmat.array[...] = sc["mats"]
        e2e_film = api.Film(ctx, 512, 512)
        h2d = pv.array.nbytes + pm.array.nbytes + pmat.array.nbytes
        d2h = pout.array.nbytes

        def e2e_step():
            s2 = api.Scene(ctx, pv.array, pm.array, pmat.array).build(stream=C_stream)
            e2e_film.reset(C_stream)
            api.render(s2, sc["camera"], st, e2e_film, C_stream)
            ctx.check(ctx.lib.crg_film_download(e2e_film.h, pout.ptr, None, None, None, None, None, C_stream))
            s2.close()

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.steps
        e2e = {"value": units_per_step * world / e2e_s / 1e6, "unit": unit, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
               "path": "crg_scene_create (pinned host geometry) + crg_scene_build + crg_film_reset + crg_render + "
                       "crg_film_download (pinned)"}
    else:
        pr = api.PinnedArray(ctx, rays_h.shape, rays_h.dtype)
        pr.array[...] = rays_h
        ph = api.PinnedArray(ctx, (units_per_step * 16,), np.uint8)
        lib = ctx.lib

        def e2e_step():
            ctx.check(lib.crg_memcpy_h2d(ctx.h, rb.ptr, pr.ptr, pr.array.nbytes, C_stream))
            ctx.check(lib.crg_intersect_closest(scene.h, rb.ptr, hb.ptr, units_per_step, C_stream))
            ctx.check(lib.crg_memcpy_d2h(ctx.h, ph.ptr, hb.ptr, units_per_step * 16, C_stream))
            ctx.check(lib.crg_stream_sync(ctx.h, C_stream))

        e2e_step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        e2e_s = (time.perf_counter() - t0) / args.steps
        e2e = {"value": units_per_step * world / e2e_s / 1e6, "unit": unit, "h2d_bytes_per_step": int(pr.array.nbytes),
               "d2h_bytes_per_step": int(units_per_step * 16), "ms_per_step": e2e_s * 1e3,
               "path": "crg_memcpy_h2d (pinned rays) + crg_intersect_closest + crg_memcpy_d2h (pinned hits)"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        if args.workload == "box":
            cv, cdt, cn = cpu_box(64)
            cpu = {"value": cv, "unit": unit, "cores": os.cpu_count(), "kind": "port",
                   "sample": f"rows 0-63 of the 512x512 64-spp box frame ({cn} samples, {cdt:.1f} s)"}
        else:
            cv, cdt, cn = cpu_soup(1 << 18)
            cpu = {"value": cv, "unit": unit, "cores": os.cpu_count(), "kind": "port",
                   "sample": f"{cn} of the 16,777,216 primary rays ({cdt:.1f} s)"}

    if rank == 0:
        line = {
            "metric": unit,
            "value": value,
            "unit": unit,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": total_s / args.steps * 1e3,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(args.workload),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "kernel": kernel, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": int(algo_bytes)},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk.summary(),
            "gpu_launches": launches_per_step * args.steps,
            **extra,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
