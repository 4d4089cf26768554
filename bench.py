#!/usr/bin/env python3
"""Benchmark: batched multi-view voxel-space render on one GB300 (or N replicas).

Workload (default "batch512"): 512 cameras over one shared 4096x4096 map pair
(u8 diamond-square heights, roughness 0.55; u32 palette colours +-12 noise),
resolutions uniform over {320x240, 640x480, 1280x720, 1920x1080, 2560x1440},
draw distance uniform in [400, 3000], yaw uniform, height 20..200 above the
local terrain maximum; reference-default depth schedule (d=0.001, z0=0,
scale=w/2), bilinear height and colour. One step renders every view once with
the persistent kernel replayed from a CUDA graph. The plain per-frame loop
(two launches per view) is timed on the same plan for comparison.

Workload "single1080": one 1920x1080 frame per step through the plain
per-frame call (fs_render_device), the walk's cameras in turn, with the
render-kernel time and the frame's gather/store roofline (frame bytes at the
HBM copy peak vs the ncu-counted gather sectors at the live-measured L2 read
rate).

Prints one JSON line (rank 0). `value` is whole-job Gpix/s with maps resident
in HBM; `e2e` is the same metric through the public C ABI with host buffers:
per step the cameras go host->device and every frame device->pinned host.
`--impl reference` times the CPU restatement of the reference path (the
oracle, OpenMP over columns, all host threads) on a bounded sample instead.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

RESOLUTIONS = [(320, 240), (640, 480), (1280, 720), (1920, 1080), (2560, 1440)]
MAP_SEED_H, MAP_SEED_C, VIEW_SEED = 7, 8, 20240601
# the metric both arms report (Gpix/s = total frame pixels / time)
METRIC = "Gpix/s (bit-exact voxel-space frames), batched multi-view"
METRIC_SINGLE = "Gpix/s (bit-exact voxel-space frames), one 1920x1080 frame per plain call"


def metric_for(workload: str) -> str:
    return METRIC_SINGLE if workload == "single1080" else METRIC


def batch_views(fs, hm, nviews: int, seed: int):
    rng = np.random.default_rng(seed)
    views = []
    for v in range(nviews):
        w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        cam = fs.gen_cameras(seed * 1000 + v, hm, 1, above=(20.0, 200.0), distance=(400.0, 3000.0),
                             screen_h=h)[0]
        views.append((cam, w, h))
    return views


def walk_views(fs, hm, seed: int):
    return [(c, 1920, 1080) for c in fs.gen_walk(seed, hm, 64, step=2.0, yaw=0.02,
                                                  above=(30.0, 120.0), distance=3000.0,
                                                  screen_h=1080)]


# the large-map workload's fused epilogue: depth shading + fog (not in the reference)
LARGE_FX = dict(effects=3, shade=0.5, fog_start=1500.0, fog_end=6000.0, fog_color=0xFFA0B0C0)


def workload_params(fs, name: str):
    return fs.default_params(**LARGE_FX) if name == "large4k" else fs.default_params()


def make_workload(fs, name: str, rank: int):
    if name == "large4k":
        hm = fs.gen_heights(MAP_SEED_H + 100, 16384, 0.6)
        cm = fs.gen_colors(MAP_SEED_C + 100, hm, 12)
        cams = fs.gen_cameras(VIEW_SEED + 17 + rank, hm, 32, above=(30.0, 150.0),
                              distance=(6000.0, 6000.0), screen_h=2160)
        return hm, cm, [(c, 3840, 2160) for c in cams], {
            "workload": "large4k: 32 views 3840x2160, D=6000, 16384^2 maps (roughness 0.6), "
                        "depth shading + fog epilogue",
            "views": 32, "map": "16384x16384 u8 heights + u32 colours (beyond L2)",
            "effects": LARGE_FX}
    if name == "batch512":
        hm = fs.gen_heights(MAP_SEED_H, 4096, 0.55)
        cm = fs.gen_colors(MAP_SEED_C, hm, 12)
        return hm, cm, batch_views(fs, hm, 512, VIEW_SEED + rank), {
            "workload": "batch512: 512 views, mixed 320x240..2560x1440, D~U[400,3000], 4096^2 maps",
            "views": 512, "map": "4096x4096 u8 heights + u32 colours", "resolutions": RESOLUTIONS}
    if name == "walk1080":
        hm = fs.gen_heights(MAP_SEED_H, 4096, 0.55)
        cm = fs.gen_colors(MAP_SEED_C, hm, 12)
        return hm, cm, walk_views(fs, hm, 9 + rank), {
            "workload": "walk1080: 64-frame walk, 1920x1080, D=3000, 4096^2 maps",
            "views": 64, "map": "4096x4096 u8 heights + u32 colours"}
    if name == "single1080":
        hm = fs.gen_heights(MAP_SEED_H, 4096, 0.55)
        cm = fs.gen_colors(MAP_SEED_C, hm, 12)
        return hm, cm, walk_views(fs, hm, 9 + rank), {
            "workload": "single1080: one 1920x1080 frame per step through the plain per-frame "
                        "call (fs_render_device), cameras of the 64-frame walk in turn, D=3000, "
                        "4096^2 maps",
            "views": 1, "map": "4096x4096 u8 heights + u32 colours"}
    raise SystemExit(f"unknown workload {name}")


def view_bytes(views, samples: int, events: int) -> dict:
    frame = sum(4 * w * h for _, w, h in views)
    return {"frame": frame, "height_gather": 4 * samples, "color_gather": 16 * events}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()
        # the timed region starts only once nvidia-smi is answering
        t0 = time.time()
        while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.005)
        self.lines.clear()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured (MEASURED_PEAKS.json)"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profiled_value(name: str, key: str):
    """A per-launch figure (`key: value` line) from the committed ncu summary
    of workload `name`, if one exists."""
    p = ROOT / "profiles" / f"render_{name}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def profiled_traffic(name: str):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    return profiled_value(name, "dram_bytes_per_launch")


def cpu_reference_rate(views, hm, cm, max_seconds: float, threads: int, params=None):
    """Oracle (CPU restatement) Gpix/s on a bounded prefix of the views."""
    import oracle
    params = params or oracle.make_params()
    px = 0
    t0 = time.perf_counter()
    used = 0
    for cam, w, h in views:
        oracle.render(cam, params, hm, cm, w, h, threads=threads)
        px += w * h
        used += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    dt = time.perf_counter() - t0
    return px / dt / 1e9, used, px, dt


def cpu_baselines(views, hm, cm, seconds: float, params=None, what: str = "views"):
    """The oracle on the host cores: OpenMP over columns on every core (the
    stand-in for a `futhark multicore` build) and one thread (for `futhark c`),
    each on a bounded prefix of the workload's views."""
    import oracle
    threads = oracle.lib().fso_max_threads()
    out = {}
    for key, nt, budget in (("multi", threads, seconds), ("single", 1, seconds / 2)):
        g, used, cpx, dt = cpu_reference_rate(views, hm, cm, budget, nt, params)
        out[key] = {"value": g, "unit": "Gpix/s", "cores": nt, "kind": "port",
                    "sample": f"first {used} {what} of the workload ({cpx} px, {dt:.1f} s), CPU "
                              "oracle (C restatement of the reference render"
                              + (", OpenMP over columns)" if nt > 1 else ", one thread)")}
    return out["multi"], out["single"]


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    import futspace_gb300 as fs
    import oracle
    hm, cm, views, cfg = make_workload(fs, args.workload, 0)
    oparams = oracle.params_from(workload_params(fs, args.workload))
    threads = oracle.lib().fso_max_threads()
    rates, pxs, dts = [], 0, 0.0
    order = list(range(len(views)))
    for step in range(args.warmup + args.steps):
        # each step: a bounded sample of the workload (views in a rotating order)
        k = (step * 7) % len(views)
        nv = 1 if args.workload == "single1080" else args.ref_views
        sample = [views[(k + i) % len(views)] for i in range(nv)]
        g, used, px, dt = cpu_reference_rate(sample, hm, cm, args.ref_seconds, threads, oparams)
        if step >= args.warmup:
            rates.append(g)
            pxs += px
            dts += dt
    value = pxs / dts / 1e9
    line = {
        "impl": "reference", "metric": metric_for(args.workload), "value": value,
        "unit": "Gpix/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * dts / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": "Gpix/s", "cores": threads, "kind": "port",
                         "sample": f"{1 if args.workload == 'single1080' else args.ref_views} "
                                   f"views per step of the {args.workload} "
                                   "workload, CPU oracle (C restatement of the reference render, "
                                   "OpenMP over columns)"},
        "e2e": {"value": value, "unit": "Gpix/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_serve(args, rank: int, world: int):
    """Serving: Poisson arrivals from 64 sessions (seeded camera walks), request
    sizes mixed as the batch512 workload, 4096^2 and 8192^2 map sets resident,
    8 GB framebuffer budget; one run per arrival rate."""
    import futspace_gb300 as fs
    import oracle

    ctx = fs.Context(int(os.environ.get("LOCAL_RANK", "0")))
    maps_np, fmaps = [], []
    for size, seed in ((4096, 7), (8192, 11)):
        hm = fs.gen_heights(seed, size, 0.55)
        cm = fs.gen_colors(seed + 1, hm, 12)
        maps_np.append((hm, cm))
        fmaps.append(fs.Map(ctx, hm, cm))
    nsess = 64
    rng = np.random.default_rng(4242 + rank)
    sess = []
    for s in range(nsess):
        w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        sess.append((w, h, s % 2, float(rng.uniform(400.0, 3000.0))))
    rates = [float(r) for r in args.serve_rates.split(",")]
    srv = fs.Server(ctx, fmaps, budget_bytes=8 << 30, nsessions=nsess, max_batch=64, slots=3,
                    max_distance=3000.0)
    results = []
    checked = bad = 0
    for ri, rate in enumerate(rates):
        n = int(rate * args.serve_seconds)
        arrivals = np.cumsum(np.random.default_rng(77 + ri).exponential(1e9 / rate, n))
        who = np.random.default_rng(99 + ri).integers(0, nsess, n)
        steps = np.bincount(who, minlength=nsess)
        walks = [fs.gen_walk(1000 * ri + s, maps_np[sess[s][2]][0], int(steps[s]) or 1, step=2.0,
                             yaw=0.02, above=(30.0, 120.0), distance=sess[s][3],
                             screen_h=sess[s][1]) for s in range(nsess)]
        pos = [0] * nsess
        reqs = (fs.Request * n)()
        sample = set(range(0, n, max(1, n // 8)))
        bufs = {}
        for i in range(n):
            s = int(who[i])
            w, h, m, _ = sess[s]
            r = reqs[i]
            r.session, r.map, r.width, r.height = s, m, w, h
            r.cam = walks[s][pos[s]]
            pos[s] += 1
            r.arrival_ns = int(arrivals[i])
            if i in sample:
                bufs[i] = fs.PinnedBuffer((h, w))
                r.host_out = bufs[i].ptr
        st = srv.run(reqs, realtime=True)
        # where the slowest requests arrived (a stall shows as one window)
        lat = np.array([(reqs[i].done_ns - reqs[i].arrival_ns) * 1e-6 for i in range(n)])
        arr_s = arrivals * 1e-9
        late = lat > 10.0 * max(st["p50_ms"], 1e-3)
        stall = {"max_ms": float(lat.max()) if n else 0.0,
                 "late_requests": int(late.sum()),
                 "late_arrivals_s": [float(arr_s[late].min()), float(arr_s[late].max())]
                 if late.any() else None}
        p = fs.default_params()
        for i, b in bufs.items():
            r = reqs[i]
            hm, cm = maps_np[r.map]
            ref = oracle.render(r.cam, oracle.params_from(p), hm, cm, r.width, r.height, threads=0)
            checked += 1
            bad += int(np.count_nonzero(ref != b.array))
            b.close()
        offered = float(np.sum([sess[int(s)][0] * sess[int(s)][1] for s in who])) / args.serve_seconds / 1e9
        results.append({"rate_req_s": rate, "requests": n, "offered_gpix_s": offered,
                        "gpix_s": st["gpix_s"], "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                        "mean_batch": st["mean_batch"], "batches": st["batches"],
                        "max_inflight": st["max_inflight"], "stall": stall,
                        "peak_arena_gb": st["peak_arena_bytes"] / 2**30, "errors": st["errors"]})
    srv.close()
    if rank == 0:
        best = max(results, key=lambda r: r["gpix_s"])
        line = {
            "metric": "serving Gpix/s with p50/p99 latency (continuous batching)",
            "value": best["gpix_s"], "unit": "Gpix/s", "n_gpus": world, "steps": len(rates),
            "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded maps, Poisson arrivals, seeded camera walks)",
            "config": {"workload": "serve: 64 sessions, mixed 320x240..2560x1440, D~U[400,3000], "
                                   "4096^2 + 8192^2 maps, 8 GB framebuffer budget",
                       "seconds_per_rate": args.serve_seconds},
            "serving": results,
            "frames_checked_vs_oracle": checked, "differing_pixels": bad,
        }
        print(json.dumps(line), flush=True)


def run_single(args, rank: int, world: int, local: int):
    """One 1920x1080 frame per step through the plain per-frame call
    (fs_render_device: depth-table kernel + render kernel), maps resident, L2
    flushed between steps, the autotuned single-frame configuration."""
    import torch
    import futspace_gb300 as fs
    from futspace_gb300 import replicas

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = f"cuda:{local}"
    ctx = fs.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=local)
    hm, cm, views, cfg = make_workload(fs, "single1080", rank)
    fmap = fs.Map(ctx, hm, cm)
    W, H = 1920, 1080
    cams = [v[0] for v in views]
    if args.tune:
        tune, tune_ms = tuple(int(x) for x in args.tune.split(",")), None
        ctx.force_tune(tune)
    else:
        tune, tune_ms = ctx.autotune_frame(fmap, cams[0], W, H, reps=5)
    out = torch.empty(W * H, dtype=torch.int32, device=dev)
    # work counters over the 64 cameras (untimed)
    ctx.stats(True)
    for c in cams:
        ctx.render_device(fmap, c, W, H, out.data_ptr())
    samples, events = ctx.stats(False)
    samples /= len(cams)
    events /= len(cams)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device=dev)
    ctx.set_option("time", 1)
    for i in range(args.warmup):
        ctx.render_device(fmap, cams[i % len(cams)], W, H, out.data_ptr())
    ctx.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches
    t_step, t_kernel = [], []
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.render_device(fmap, cams[i % len(cams)], W, H, out.data_ptr())
        b.record(stream)
        b.synchronize()
        t_step.append(a.elapsed_time(b))
        t_kernel.append(ctx.kernel_ms())
    gpu_launches = ctx.launches - launches0
    clk = clocks.stop()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ctx.set_option("time", 0)

    # end to end through the C ABI with a host buffer: fs_render renders and
    # copies the frame to pinned host memory, then waits for it
    e2e = None
    if not args.no_e2e:
        host = fs.PinnedBuffer((H, W))
        t_e2e = []
        for i in range(args.warmup + args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.render(fmap, cams[i % len(cams)], W, H, out=host.array)
            b.record(stream)
            b.synchronize()
            if i >= args.warmup:
                t_e2e.append(a.elapsed_time(b))
        e2e_ms = float(np.mean(t_e2e))
        e2e = {"value": W * H / e2e_ms / 1e6, "unit": "Gpix/s",
               # the camera travels in the launch parameters (one view record)
               "h2d_bytes_per_step": 128, "d2h_bytes_per_step": 4 * W * H,
               "ms_per_step": e2e_ms}
        host.close()

    ms = float(np.mean(t_step))
    agg = replicas.aggregate(W * H, ms, dist=dist, device=dev)
    k_ms = float(np.mean(t_kernel))
    peaks = measured_peaks()
    l2_gbs = max(ctx.measure_l2_read_gbs() for _ in range(3))
    vb = {"frame": 4 * W * H, "height_gather": 4 * samples, "color_gather": 16 * events}
    alg = vb["frame"] + vb["height_gather"] + vb["color_gather"]
    achieved = alg / (k_ms * 1e-3) / 1e9
    n = fs.num_depths(cams[0].distance)
    # the gather/store roofline of one frame: the slower of the frame bytes at
    # the HBM copy rate and the gathers' L2 read sectors (ncu, committed
    # summary; else the algorithmic gather bytes) at the measured L2 read rate
    sectors = profiled_value("single1080", "l2_read_sectors_per_launch")
    gather_bytes = 32 * sectors if sectors else vb["height_gather"] + vb["color_gather"]
    store_us = 4 * W * H / (peaks["hbm_gbs"] * 1e3)
    gather_us = gather_bytes / (l2_gbs * 1e3)
    bound_us = max(store_us, gather_us)
    # the same with the reference's full gather work, every depth sample of
    # every column at 20 B (a 4-byte height quad, four colour texels): larger
    # than what this kernel reads, which skips samples
    full_us = max(store_us, n * W * 20 / (l2_gbs * 1e3))

    cpu = cpu1 = None
    if rank == 0 and args.cpu_seconds > 0:
        cpu, cpu1 = cpu_baselines(views, hm, cm, args.cpu_seconds, what="frames")
    if rank == 0:
        line = {
            "metric": METRIC_SINGLE,
            "value": agg["gpix_s"], "unit": "Gpix/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": agg["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded diamond-square maps and camera walk)",
            "config": {**cfg, "l2": "flushed between timed steps (256 MB write)",
                       "tune": {"tile_width": tune[0], "threads_or_lanes_per_column": tune[1],
                                "depth_per_thread": tune[2], "stage": tune[3]},
                       "autotune_ms": tune_ms},
            "latency_ms": {"p50": float(np.percentile(t_step, 50)),
                           "p99": float(np.percentile(t_step, 99))},
            "frames_per_s": world / agg["ms"] * 1e3,
            "work": {"depth_samples_per_frame": samples, "full_depth_samples": n * W,
                     "events_coloured_per_frame": events},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                         "traffic": profiled_traffic("single1080"),
                         "peak_source": peaks["source"],
                         "kernel": "the kernels of one plain call (depth table + render, "
                                   "the render a programmatic dependent launch)",
                         "kernel_ms": k_ms,
                         "bytes_per_launch": vb},
            "gather_store_roofline": {"store_us": store_us, "gather_us": gather_us,
                                      "gather_bytes": gather_bytes,
                                      "gather_bytes_source": "ncu L2 read sectors x 32"
                                      if sectors else "algorithmic gather bytes",
                                      "l2_read_gbs_measured": l2_gbs, "bound_us": bound_us,
                                      "kernel_us": k_ms * 1e3,
                                      "frac": bound_us / (k_ms * 1e3),
                                      "bound_us_full_work": full_us,
                                      "frac_full_work": full_us / (k_ms * 1e3)},
            "clocks": clk,
            "e2e": e2e,
            "gpu_launches": gpu_launches,
            "cpu_baseline": cpu,
            "cpu_baseline_one_thread": cpu1,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch512",
                    choices=["batch512", "walk1080", "large4k", "single1080", "serve"])
    ap.add_argument("--serve-rates", default="1000,5000,10000,20000")
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tune", default="",
                    help="pin the plan's kernel configuration: tile_width,lanes_per_column,"
                         "depth_per_lane,stage (skips the autotuner)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-groups", type=int, default=8,
                    help="view groups of the pipelined render + download in the e2e timing")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-views", type=int, default=4)
    ap.add_argument("--ref-seconds", type=float, default=20.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "serve":
        run_serve(args, rank, world)
        return
    if args.workload == "single1080":
        run_single(args, rank, world, local)
        return

    import torch
    import futspace_gb300 as fs
    from futspace_gb300 import replicas

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    ctx = fs.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=local)
    hm, cm, views, cfg = make_workload(fs, args.workload, rank)
    fmap = fs.Map(ctx, hm, cm)
    wparams = workload_params(fs, args.workload)
    plan = fs.Plan(ctx, [fmap], views, params=wparams)
    tune_info = None
    if args.tune:
        plan.set_tune(*[int(x) for x in args.tune.split(",")])
    elif not args.no_autotune:
        tune_info = plan.autotune(reps=3)
    tune = plan.get_tune()
    px = sum(w * h for _, w, h in views)

    # L2 flush buffer (larger than the 129 MB L2), written between timed steps
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device=f"cuda:{local}")

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.fill_(1)

    # work counters (untimed): evaluated depth samples and coloured events
    ctx.stats(True)
    plan.run()
    samples, events = ctx.stats(False)

    def timed(fn, steps, kernel=None):
        times = []
        for _ in range(steps):
            flush_l2()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
            if kernel is not None:
                kernel.append(plan.kernel_ms())
        return times

    for _ in range(args.warmup):
        plan.run()
    ctx.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches
    t_kernel: list[float] = []
    t_batch = timed(plan.run, args.steps, t_kernel)
    gpu_launches = ctx.launches - launches0
    clk = clocks.stop()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    t_plain = []
    if not args.no_plain:
        # the per-frame loop runs each resolution with its own autotuned configuration
        seen = set()
        for cam, w, h in views:
            if (w, h) not in seen:
                seen.add((w, h))
                ctx.autotune_frame(fmap, cam, w, h, params=wparams, reps=3)
        plan.run_per_view()
        ctx.sync()
        t_plain = timed(plan.run_per_view, max(3, args.steps // 2))

    # end to end through the C ABI: cameras host->device, then the pipelined
    # render + download (fs_plan_run_download): frames -> pinned host memory
    e2e = None
    if not args.no_e2e:
        host = torch.empty(plan.total_pixels, dtype=torch.int32, pin_memory=True)
        cams = [v[0] for v in views]
        t_e2e = []
        for i in range(args.warmup + max(3, args.steps // 2)):
            flush_l2()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            plan.set_cameras(cams)
            plan.run_download(host.numpy().view(np.uint32), groups=args.e2e_groups)
            b.record(stream)
            b.synchronize()
            if i >= args.warmup:
                t_e2e.append(a.elapsed_time(b))
        e2e_ms = float(np.mean(t_e2e))
        e2e = {"value": px / e2e_ms / 1e6, "unit": "Gpix/s",
               "h2d_bytes_per_step": 96 * len(views),  # one 96-byte view record per camera
               "d2h_bytes_per_step": 4 * plan.total_pixels,
               "ms_per_step": e2e_ms, "groups": args.e2e_groups}

    ms = float(np.mean(t_batch))
    # replicas: every rank renders its own views; sum pixels, slowest rank's time
    agg = replicas.aggregate(px, ms, dist=dist, device=f"cuda:{local}")
    ms_max = agg["ms"]
    value = agg["gpix_s"]

    peaks = measured_peaks()
    vb = view_bytes(views, samples, events)
    alg = vb["frame"] + vb["height_gather"] + vb["color_gather"]
    # the dominant kernel's own device time: events recorded inside the graph
    # around the persistent render kernel, read back after every timed step
    k_ms = float(np.mean(t_kernel)) if t_kernel else ms
    achieved = alg / (k_ms * 1e-3) / 1e9
    traffic = profiled_traffic(args.workload)
    # gather/store roofline of the launch: the slower of the frame bytes at the
    # HBM copy peak and the gathers' L2 read sectors (committed ncu summary of
    # this workload; else the algorithmic gather bytes) at the live L2 read rate
    l2_gbs = max(ctx.measure_l2_read_gbs() for _ in range(3))
    sectors = profiled_value(args.workload, "l2_read_sectors_per_launch")
    gather_bytes = 32 * sectors if sectors else vb["height_gather"] + vb["color_gather"]
    gs_store_ms = vb["frame"] / (peaks["hbm_gbs"] * 1e6)
    gs_gather_ms = gather_bytes / (l2_gbs * 1e6)
    gs_bound_ms = max(gs_store_ms, gs_gather_ms)

    cpu = cpu1 = None
    if rank == 0 and args.cpu_seconds > 0:
        import oracle
        cpu, cpu1 = cpu_baselines(views, hm, cm, args.cpu_seconds, oracle.params_from(wparams))

    if rank == 0:
        full_s = sum(fs.num_depths(v[0].distance) * v[1] for v in views)
        line = {
            "metric": METRIC,
            "value": value, "unit": "Gpix/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded diamond-square maps and cameras)",
            "config": {**cfg, "l2": "flushed between timed steps (256 MB write)",
                       "tune": {"tile_width": tune[0], "lanes_per_column": tune[1],
                                "depth_per_lane": tune[2], "stage": tune[3],
                                "persistent_ctas": tune[4]}},
            "latency_ms": {"p50": float(np.percentile(t_batch, 50)),
                           "p99": float(np.percentile(t_batch, 99))},
            "plain_per_frame": None if not t_plain else {
                "value": px / float(np.mean(t_plain)) / 1e6, "unit": "Gpix/s",
                "ms_per_step": float(np.mean(t_plain)),
                "p50_ms": float(np.percentile(t_plain, 50)),
                "p99_ms": float(np.percentile(t_plain, 99)),
                "launches_per_step": 2 * len(views)},
            "batched_over_plain": None if not t_plain else float(np.mean(t_plain)) / ms,
            "frames_per_s": len(views) * world / ms_max * 1e3,
            "work": {"depth_samples": samples, "full_depth_samples": full_s,
                     "events_coloured": events},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                         "traffic": traffic, "peak_source": peaks["source"],
                         "kernel": "render_kernel (persistent, one launch per step)",
                         "kernel_ms": k_ms, "bytes_per_launch": vb},
            "gather_store_roofline": {"store_ms": gs_store_ms, "gather_ms": gs_gather_ms,
                                      "gather_bytes": gather_bytes,
                                      "gather_bytes_source": "ncu L2 read sectors x 32"
                                      if sectors else "algorithmic gather bytes",
                                      "l2_read_gbs_measured": l2_gbs, "bound_ms": gs_bound_ms,
                                      "kernel_ms": k_ms, "frac": gs_bound_ms / k_ms},
            "clocks": clk,
            "e2e": e2e,
            "gpu_launches": gpu_launches,
            "cpu_baseline": cpu,
            "cpu_baseline_one_thread": cpu1,
        }
        if tune_info:
            line["config"]["autotune_ms"] = tune_info[1]
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
