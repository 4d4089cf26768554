#!/usr/bin/env python3
"""Benchmark: batched multi-view voxel-space render on one GB300 (or N replicas).

Workload (default "batch512"): 512 cameras over one shared 4096x4096 map pair
(u8 diamond-square heights, roughness 0.55; u32 palette colours +-12 noise),
resolutions uniform over {320x240, 640x480, 1280x720, 1920x1080, 2560x1440},
draw distance uniform in [400, 3000], yaw uniform, height 20..200 above the
local terrain maximum; reference-default depth schedule (d=0.001, z0=0,
scale=w/2), bilinear height and colour. One step renders every view once with
the persistent kernel replayed from a CUDA graph. The plain per-frame loop
(two launches per view) is timed on the same plan for comparison. After the
timed region a stratified sample of the frames (per resolution the views with
the largest and the smallest draw distance) is diffed against the CPU oracle.

The default run also times three shorter workloads and reports them under
`extra_workloads` (single 1920x1080 frames through the plain call, the 64-frame
1080p walk as one plan, and 32 4K views over 16384^2 maps with the shading/fog
epilogue), each with its own roofline and oracle diff.

Workload "single1080": one 1920x1080 frame per step through the plain
per-frame call (fs_render_device), the walk's cameras in turn.

Roofline (`roofline`): the kernel's bound is the slower of the frame stores at
the HBM copy peak and the reference's full gather work -- every depth sample of
every column at 20 B (one 4-byte height quad, four 4-byte colour texels) -- at
the L2 read rate (maps that fit in L2) or the HBM copy peak (maps beyond L2).
`frac` = that time / the render kernel's CUDA-event time. The same with only
the depth samples the kernel evaluated is `roofline.effective`.

Prints one JSON line (rank 0). `value` is whole-job Gpix/s with maps resident
in HBM; `e2e` is the same metric through the public C ABI with host buffers:
per step the cameras go host->device and every frame device->pinned host.
`--impl reference` times the CPU restatement of the reference path (the
oracle, OpenMP over columns, all host threads) on a resolution-stratified
sample instead, with inputs made by the oracle-side generators (the product
library is not loaded).
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
L2_POLICY = "GPU arm: L2 flushed between timed steps (256 MB write)"
L2_POLICY_SINGLE = ("GPU arm: L2 flushed between timed steps (1 GB write, long enough that "
                    "the call's launches are queued before the GPU reaches them)")
L2_BYTES = 126 << 20  # GB300 L2 capacity (cudaDevAttrL2CacheSize)
GATHER_BYTES_PER_SAMPLE = 20  # one 4-byte height quad + four 4-byte colour texels


def metric_for(workload: str) -> str:
    return METRIC_SINGLE if workload == "single1080" else METRIC


class ProductGen:
    """The product library's seeded generators under the oracle-side names
    (oracle.gen makes the same bytes without loading the library)."""

    def __init__(self, fs):
        self.fs = fs

    def heights(self, seed, size, roughness):
        return self.fs.gen_heights(seed, size, roughness)

    def colors(self, seed, hm, noise):
        return self.fs.gen_colors(seed, hm, noise)

    def cameras(self, seed, hm, count, **kw):
        return self.fs.gen_cameras(seed, hm, count, **kw)

    def walk(self, seed, hm, count, **kw):
        return self.fs.gen_walk(seed, hm, count, **kw)


def batch_views(gen, hm, nviews: int, seed: int):
    rng = np.random.default_rng(seed)
    views = []
    for v in range(nviews):
        w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        cam = gen.cameras(seed * 1000 + v, hm, 1, above=(20.0, 200.0), distance=(400.0, 3000.0),
                          screen_h=h)[0]
        views.append((cam, w, h))
    return views


def walk_views(gen, hm, seed: int):
    return [(c, 1920, 1080) for c in gen.walk(seed, hm, 64, step=2.0, yaw=0.02,
                                              above=(30.0, 120.0), distance=3000.0,
                                              screen_h=1080)]


# the large-map workload's fused epilogue: depth shading + fog (not in the reference)
LARGE_FX = dict(effects=3, shade=0.5, fog_start=1500.0, fog_end=6000.0, fog_color=0xFFA0B0C0)


def make_workload(gen, name: str, rank: int):
    """(heights, colours, [(camera, W, H)], config). The config dict is the
    same in both arms."""
    if name == "large4k":
        hm = gen.heights(MAP_SEED_H + 100, 16384, 0.6)
        cm = gen.colors(MAP_SEED_C + 100, hm, 12)
        cams = gen.cameras(VIEW_SEED + 17 + rank, hm, 32, above=(30.0, 150.0),
                           distance=(6000.0, 6000.0), screen_h=2160)
        return hm, cm, [(c, 3840, 2160) for c in cams], {
            "workload": "large4k: 32 views 3840x2160, D=6000, 16384^2 maps (roughness 0.6), "
                        "depth shading + fog epilogue",
            "views": 32, "map": "16384x16384 u8 heights + u32 colours (beyond L2)",
            "effects": LARGE_FX, "l2": L2_POLICY}
    hm = gen.heights(MAP_SEED_H, 4096, 0.55)
    cm = gen.colors(MAP_SEED_C, hm, 12)
    if name == "batch512":
        return hm, cm, batch_views(gen, hm, 512, VIEW_SEED + rank), {
            "workload": "batch512: 512 views, mixed 320x240..2560x1440, D~U[400,3000], 4096^2 maps",
            "views": 512, "map": "4096x4096 u8 heights + u32 colours",
            "resolutions": RESOLUTIONS, "l2": L2_POLICY}
    if name == "walk1080":
        return hm, cm, walk_views(gen, hm, 9 + rank), {
            "workload": "walk1080: 64-frame walk, 1920x1080, D=3000, 4096^2 maps",
            "views": 64, "map": "4096x4096 u8 heights + u32 colours", "l2": L2_POLICY}
    if name == "single1080":
        return hm, cm, walk_views(gen, hm, 9 + rank), {
            "workload": "single1080: one 1920x1080 frame per step through the plain per-frame "
                        "call (fs_render_device), cameras of the 64-frame walk in turn, D=3000, "
                        "4096^2 maps",
            "views": 1, "map": "4096x4096 u8 heights + u32 colours", "l2": L2_POLICY_SINGLE}
    raise SystemExit(f"unknown workload {name}")


def oracle_params(name: str):
    import oracle
    return oracle.make_params(**LARGE_FX) if name == "large4k" else oracle.make_params()


def cam_field(cam, k):
    return cam[k] if isinstance(cam, dict) else getattr(cam, k)


def by_resolution(views) -> dict:
    groups: dict = {}
    for i, (_, w, h) in enumerate(views):
        groups.setdefault((w, h), []).append(i)
    return groups


def check_sample(views) -> list[int]:
    """Per resolution, the views with the largest and the smallest draw
    distance, plus the middle and the last view of that resolution when the
    distances are all equal (at least two views per resolution)."""
    out = []
    for idxs in by_resolution(views).values():
        ds = [cam_field(views[i][0], "distance") for i in idxs]
        pick = [int(np.argmax(ds)), int(np.argmin(ds))]
        if pick[0] == pick[1]:
            pick += [len(idxs) // 2, len(idxs) - 1]
        for j in pick:
            if idxs[j] not in out:
                out.append(idxs[j])
    return sorted(out)


def oracle_diff(frames: dict, views, hm, cm, oparams) -> dict:
    """Differing pixels of GPU frames {view index: [H][W] u32} against the oracle."""
    import oracle
    bad = 0
    for i, got in frames.items():
        cam, w, h = views[i]
        ref = oracle.render(cam, oparams, hm, cm, w, h, threads=0)
        bad += int(np.count_nonzero(ref != got))
    return {"frames_checked_vs_oracle": len(frames), "differing_pixels": bad,
            "checked_views": sorted(frames), "check": "per resolution the views with the "
            "largest and smallest draw distance (at least two views), after the timed region"}


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
        # a timed region shorter than the sampling interval: wait for one sample
        t0 = time.time()
        while not self.lines and time.time() - t0 < 1.0 and self.proc.poll() is None:
            time.sleep(0.005)
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
    return {"hbm_gbs": 6800.0, "source": "fallback (6.8 TB/s)"}


def capture_figures(name: str, tune) -> dict:
    """Per-launch ncu figures from the committed summary of workload `name`:
    its `capture TW,LC,U,STAGE: key value ...` line for the kernel
    configuration this run uses, else {} -- a capture of another configuration
    says nothing about this launch."""
    p = ROOT / "profiles" / f"render_{name}.md"
    if not p.exists():
        return {}
    want = ",".join(str(int(x)) for x in tune[:4])
    for line in p.read_text().splitlines():
        if not line.startswith("capture ") or ":" not in line:
            continue
        head, body = line[len("capture "):].split(":", 1)
        if head.replace(" ", "") != want:
            continue
        out = {"capture_tune": want}
        words = body.split()
        for k, v in zip(words[0::2], words[1::2]):
            try:
                out[k] = float(v)
            except ValueError:
                pass
        return out
    return {}


def roofline(frame_bytes: int, s_full: int, s_eff: int, kernel_ms: float, hbm_gbs: float,
             l2_gbs: float, maps_fit_l2: bool, hbm_source: str, captured: dict,
             kernel: str, events: int | None = None) -> dict:
    """T_roof = max(frame bytes / HBM copy peak, 20 B x depth samples / gather
    peak); frac = T_roof / kernel time. The gather peak is the L2 read rate for
    maps that fit in L2, else the HBM copy peak (the gathers fall to DRAM)."""
    g_peak = l2_gbs if maps_fit_l2 else hbm_gbs
    t_frame = frame_bytes / (hbm_gbs * 1e6)  # ms
    t_full = GATHER_BYTES_PER_SAMPLE * s_full / (g_peak * 1e6)
    t_eff = GATHER_BYTES_PER_SAMPLE * s_eff / (g_peak * 1e6)
    gather_dominates = t_full >= t_frame
    alg = GATHER_BYTES_PER_SAMPLE * s_full if gather_dominates else frame_bytes
    peak = g_peak if gather_dominates else hbm_gbs
    achieved = alg / (kernel_ms * 1e-3) / 1e9
    bound = ("l2" if maps_fit_l2 else "hbm") if gather_dominates else "hbm"
    src_l2 = (f"L2 read rate: builder probe in this run (fs_measure_l2_read_gbs, "
              f"{l2_gbs:.0f} GB/s)")
    out = {
        "bound": bound, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": captured.get("dram_bytes_per_launch"),
        "traffic_source": ("ncu capture of this kernel configuration (profiles/), "
                           f"tune {captured['capture_tune']}" if captured else
                           "none: no committed ncu capture of this kernel configuration"),
        "form": "max(frame bytes / HBM copy peak, 20 B x full depth samples / gather peak) "
                "/ kernel time",
        "peak_source": f"HBM: {hbm_source}; " + (src_l2 if maps_fit_l2 else
                                                  "gathers: maps beyond L2, HBM copy peak"),
        "kernel": kernel, "kernel_ms": kernel_ms,
        "t_roof_ms": max(t_frame, t_full), "t_frame_ms": t_frame, "t_gather_full_ms": t_full,
        "frame_bytes": frame_bytes, "full_depth_samples": s_full,
        "gather_bytes_full": GATHER_BYTES_PER_SAMPLE * s_full,
        "l2_read_gbs_measured": l2_gbs, "hbm_gbs": hbm_gbs,
        "effective": {"depth_samples": s_eff, "t_roof_ms": max(t_frame, t_eff),
                      "frac": max(t_frame, t_eff) / kernel_ms,
                      "note": "the depth samples the kernel evaluated (after exact skips "
                              "and early exit)"},
    }
    if events is not None:
        # the earlier form: the bytes this kernel's work reads and writes (frame,
        # a 4-byte height quad per evaluated sample, four colour texels per
        # event) against the HBM copy peak
        alg = frame_bytes + 4 * s_eff + 16 * events
        out["hbm_copy_form"] = {"bytes": alg, "achieved": alg / (kernel_ms * 1e-3) / 1e9,
                                "frac": alg / (kernel_ms * 1e-3) / 1e9 / hbm_gbs}
    sectors = captured.get("l2_read_sectors_per_launch")
    if sectors:
        t_sec = 32 * sectors / (l2_gbs * 1e6)
        out["ncu_sector_form"] = {"l2_read_sectors": sectors, "t_roof_ms": max(t_frame, t_sec),
                                  "frac": max(t_frame, t_sec) / kernel_ms}
    return out


def cpu_rate_stratified(views, hm, cm, oparams, threads: int, budget_s: float) -> dict:
    """The oracle on the host cores, in rounds of one view per resolution
    (rotating through each resolution's views) until the time budget is spent.
    The rate is the workload's own mix: count_r views of resolution r at that
    resolution's mean time per view."""
    import oracle
    groups = by_resolution(views)
    t_sum = {r: 0.0 for r in groups}
    n_done = {r: 0 for r in groups}
    t0 = time.perf_counter()
    rnd = 0
    while True:
        for r, idxs in groups.items():
            cam, w, h = views[idxs[rnd % len(idxs)]]
            t = time.perf_counter()
            oracle.render(cam, oparams, hm, cm, w, h, threads=threads)
            t_sum[r] += time.perf_counter() - t
            n_done[r] += 1
        rnd += 1
        if time.perf_counter() - t0 > budget_s:
            break
    px = sum(len(idxs) * w * h for (w, h), idxs in groups.items())
    t = sum(len(idxs) * t_sum[r] / n_done[r] for r, idxs in groups.items())
    rendered = sum(n_done.values())
    return {"value": px / t / 1e9, "unit": "Gpix/s", "cores": threads, "kind": "port",
            "sample": f"{rnd} rounds of one view per resolution ({rendered} views, "
                      f"{time.perf_counter() - t0:.1f} s), rate weighted by the workload's "
                      "views per resolution; CPU oracle (C restatement of the reference render"
                      + (", OpenMP over columns)" if threads > 1 else ", one thread)")}


def cpu_baselines(views, hm, cm, seconds: float, oparams):
    """The oracle on all host cores (the stand-in for a `futhark multicore`
    build) and on one thread (for `futhark c`)."""
    import oracle
    threads = oracle.lib().fso_max_threads()
    return (cpu_rate_stratified(views, hm, cm, oparams, threads, seconds),
            cpu_rate_stratified(views, hm, cm, oparams, 1, seconds / 2))


def run_reference(args, rank: int, world: int):
    """The CPU reference arm: the oracle port on every host thread, each step
    one view per resolution of the workload (a rotating stratified sample),
    the rate weighted by the workload's own resolution mix. Inputs come from
    the oracle-side generators, so the product library is never loaded."""
    if rank != 0:
        return
    import oracle
    from oracle import gen
    hm, cm, views, cfg = make_workload(gen, args.workload, 0)
    oparams = oracle_params(args.workload)
    threads = oracle.lib().fso_max_threads()
    groups = by_resolution(views)
    t_sum = {r: 0.0 for r in groups}
    n_done = {r: 0 for r in groups}
    step_ms = []
    for step in range(args.warmup + args.steps):
        t_step = 0.0
        for r, idxs in groups.items():
            cam, w, h = views[idxs[step % len(idxs)]]
            t = time.perf_counter()
            oracle.render(cam, oparams, hm, cm, w, h, threads=threads)
            dt = time.perf_counter() - t
            t_step += dt
            if step >= args.warmup:
                t_sum[r] += dt
                n_done[r] += 1
        if step >= args.warmup:
            step_ms.append(1000.0 * t_step)
    px = sum(len(idxs) * w * h for (w, h), idxs in groups.items())
    t = sum(len(idxs) * t_sum[r] / max(1, n_done[r]) for r, idxs in groups.items())
    value = px / t / 1e9
    sample = (f"each step one view per resolution ({len(groups)} views, rotating through each "
              "resolution's views), the rate weighted by the workload's views per resolution; "
              "CPU oracle (C restatement of the reference render, OpenMP over columns), inputs "
              "from the oracle-side generators")
    line = {
        "impl": "reference", "metric": metric_for(args.workload), "value": value,
        "unit": "Gpix/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(step_ms)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "cpu_baseline": {"value": value, "unit": "Gpix/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "Gpix/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _read(path: str):
    try:
        return Path(path).read_text().strip()
    except OSError:
        return None


def cgroup_cpu_stat() -> dict:
    """The process's cgroup CPU counters (cgroup v2 cpu.stat), {} if absent."""
    out = {}
    try:
        for line in Path("/sys/fs/cgroup/cpu.stat").read_text().splitlines():
            k, v = line.split()
            out[k] = int(v)
    except (OSError, ValueError):
        pass
    return out


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
        cg0 = cgroup_cpu_stat()
        st = srv.run(reqs, realtime=True)
        cg1 = cgroup_cpu_stat()
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
                        "loop_diagnostics": {
                            "max_call_ms": st["max_call_ms"], "max_call_site": st["max_call_site"],
                            "max_sleep_ms": st["max_sleep_ms"], "max_host_ms": st["max_host_ms"],
                            "max_batch_gpu_ms": st["max_batch_gpu_ms"],
                            "max_batch_gpu_at_s": st["max_batch_gpu_at_ns"] * 1e-9,
                            "max_host_at_s": st["max_host_at_ns"] * 1e-9,
                            "involuntary_switches": st["involuntary_switches"],
                            "voluntary_switches": st["voluntary_switches"],
                            "cgroup_throttled": {k: cg1[k] - cg0.get(k, 0) for k in cg1
                                                 if k.startswith(("nr_throttled", "throttled"))}},
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
            "host": {"cpus": os.cpu_count(), "cgroup_cpu_max": _read("/sys/fs/cgroup/cpu.max")},
        }
        print(json.dumps(line), flush=True)


def single_leg(fs, ctx, args, rank: int, world: int, local: int, steps: int, warmup: int,
               dist=None, with_cpu: bool = True, with_e2e: bool = True) -> dict:
    """One 1920x1080 frame per step through the plain per-frame call
    (fs_render_device: depth-table kernel + render kernel), maps resident, L2
    flushed between steps, the autotuned single-frame configuration."""
    import torch
    from futspace_gb300 import replicas

    dev = f"cuda:{local}"
    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=local)
    hm, cm, views, cfg = make_workload(ProductGen(fs), "single1080", rank)
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
    # L2 flush between frames: 1 GB, whose write outlasts the host's submission of
    # the next call (Python and ctypes overhead included), so the events bracket
    # device execution rather than the GPU waiting for the host's second launch
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.int32, device=dev)
    ctx.set_option("time", 1)
    for i in range(warmup):
        ctx.render_device(fmap, cams[i % len(cams)], W, H, out.data_ptr())
    ctx.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches
    t_step, t_kernel = [], []
    for i in range(steps):
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
    # bit-exactness: the last timed frame and two more of the walk
    frames = {(steps - 1) % len(cams): out.cpu().numpy().view(np.uint32).reshape(H, W).copy()}
    for i in (0, len(cams) // 2):
        if i not in frames:
            ctx.render_device(fmap, cams[i], W, H, out.data_ptr())
            ctx.sync()
            frames[i] = out.cpu().numpy().view(np.uint32).reshape(H, W).copy()
    parity = oracle_diff(frames, views, hm, cm, oracle_params("single1080"))
    parity["check"] = "the last timed frame and walk frames 0 and 32, after the timed region"

    # end to end through the C ABI with a host buffer: fs_render renders and
    # copies the frame to pinned host memory, then waits for it
    e2e = None
    if with_e2e:
        host = fs.PinnedBuffer((H, W))
        t_e2e = []
        for i in range(warmup + steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.render(fmap, cams[i % len(cams)], W, H, out=host.array)
            b.record(stream)
            b.synchronize()
            if i >= warmup:
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
    n = fs.num_depths(cams[0].distance)
    rl = roofline(4 * W * H, n * W, int(samples), k_ms, peaks["hbm_gbs"], l2_gbs, True,
                  peaks["source"], capture_figures("single1080", tune),
                  "the kernels of one plain call (depth table + render, the render a "
                  "programmatic dependent launch)", int(events))
    cpu = cpu1 = None
    if rank == 0 and with_cpu and args.cpu_seconds > 0:
        cpu, cpu1 = cpu_baselines(views, hm, cm, args.cpu_seconds, oracle_params("single1080"))
    fmap.close()
    ctx.force_tune(None)
    return {
        "metric": METRIC_SINGLE,
        "value": agg["gpix_s"], "unit": "Gpix/s", "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": agg["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded diamond-square maps and camera walk)",
        "config": cfg,
        "tune": {"tile_width": tune[0], "threads_or_lanes_per_column": tune[1],
                 "depth_per_thread": tune[2], "stage": tune[3], "autotune_ms": tune_ms},
        "latency_ms": {"p50": float(np.percentile(t_step, 50)),
                       "p99": float(np.percentile(t_step, 99))},
        "frames_per_s": world / agg["ms"] * 1e3,
        "work": {"depth_samples_per_frame": samples, "full_depth_samples": n * W,
                 "events_coloured_per_frame": events},
        "roofline": rl,
        **parity,
        "clocks": clk,
        "e2e": e2e,
        "gpu_launches": gpu_launches,
        "cpu_baseline": cpu,
        "cpu_baseline_one_thread": cpu1,
    }


def plan_leg(fs, ctx, args, name: str, rank: int, world: int, local: int, steps: int,
             warmup: int, dist=None, headline: bool = True) -> dict:
    """One workload as a batch plan: every view per step with the persistent
    kernel replayed from a CUDA graph; with `headline`, also the plain
    per-frame loop, the end-to-end time and the CPU baselines."""
    import torch
    from futspace_gb300 import replicas

    stream = torch.cuda.ExternalStream(ctx.stream_handle, device=local)
    hm, cm, views, cfg = make_workload(ProductGen(fs), name, rank)
    fmap = fs.Map(ctx, hm, cm)
    wparams = fs.default_params(**LARGE_FX) if name == "large4k" else fs.default_params()
    plan = fs.Plan(ctx, [fmap], views, params=wparams)
    tune_info = None
    if args.tune and headline:
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

    def timed(fn, nsteps, kernel=None):
        times = []
        for _ in range(nsteps):
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

    for _ in range(warmup):
        plan.run()
    ctx.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches
    t_kernel: list[float] = []
    t_batch = timed(plan.run, steps, t_kernel)
    gpu_launches = ctx.launches - launches0
    clk = clocks.stop()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    # bit-exactness of the frames of the last timed step (untimed)
    host = torch.empty(plan.total_pixels, dtype=torch.int32, pin_memory=True)
    flat = plan.download(host.numpy().view(np.uint32))
    idx = check_sample(views)
    frames = {}
    for i in idx:
        _, w, h = views[i]
        o = plan.frame_offset(i)
        frames[i] = flat[o:o + w * h].reshape(h, w).copy()
    parity = oracle_diff(frames, views, hm, cm, oracle_params(name))

    t_plain = []
    if headline and not args.no_plain:
        # the per-frame loop runs each resolution with its own autotuned configuration
        seen = set()
        for cam, w, h in views:
            if (w, h) not in seen:
                seen.add((w, h))
                ctx.autotune_frame(fmap, cam, w, h, params=wparams, reps=3)
        plan.run_per_view()
        ctx.sync()
        t_plain = timed(plan.run_per_view, max(3, steps // 2))

    # end to end through the C ABI: cameras host->device, then the pipelined
    # render + download (fs_plan_run_download): frames -> pinned host memory
    e2e = None
    if headline and not args.no_e2e:
        cams = [v[0] for v in views]
        t_e2e = []
        for i in range(warmup + max(3, steps // 2)):
            flush_l2()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            plan.set_cameras(cams)
            plan.run_download(host.numpy().view(np.uint32), groups=args.e2e_groups)
            b.record(stream)
            b.synchronize()
            if i >= warmup:
                t_e2e.append(a.elapsed_time(b))
        e2e_ms = float(np.mean(t_e2e))
        # the rows below each view's all-sky rows crossed the link (plus a
        # 4-byte row count per view); the host wrote the sky rows
        copied, filled = plan.download_bytes()
        # the host frames of the last step against the device's frames
        # (whose sample was diffed against the oracle above)
        dev_flat = plan.download()
        e2e_bad = int(np.count_nonzero(dev_flat != host.numpy().view(np.uint32)))
        del dev_flat
        e2e = {"value": px / e2e_ms / 1e6, "unit": "Gpix/s",
               "h2d_bytes_per_step": 96 * len(views),  # one 96-byte view record per camera
               "d2h_bytes_per_step": copied,
               "host_written_sky_bytes_per_step": filled,
               "frame_bytes_per_step": 4 * plan.total_pixels,
               "differing_pixels_vs_device_frames": e2e_bad,
               "ms_per_step": e2e_ms, "groups": args.e2e_groups}
        # for comparison: the device-to-host copy of the whole frames alone
        # (fs_plan_download into the same pinned buffer)
        t_copy = []
        for i in range(4):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            plan.download(host.numpy().view(np.uint32))
            b.record(stream)
            b.synchronize()
            if i:
                t_copy.append(a.elapsed_time(b))
        copy_ms = float(np.median(t_copy))
        e2e["host_link"] = {"full_copy_ms": copy_ms,
                            "gbs": 4 * plan.total_pixels / copy_ms / 1e6,
                            "full_copy_gpix_s": px / copy_ms / 1e6,
                            "e2e_over_full_copy": copy_ms / e2e_ms}

    # the kernel forms on this plan, one configuration each (the autotuner
    # times every compiled configuration; these are the best-known of each
    # form): direct painting, the shared-memory stage with TMA row stores, the
    # cooperative tile
    forms = None
    if headline and not args.no_forms and world == 1:
        forms = {}
        for label, t in (("direct painting (64,2,4,0)", (64, 2, 4, 0)),
                         ("staged, TMA row stores (8,32,2,1)", (8, 32, 2, 1)),
                         ("cooperative tile (8,64,8,2)", (8, 64, 8, 2))):
            try:
                plan.set_tune(*t)
            except fs.FsError as e:
                forms[label] = f"unsupported: {e}"
                continue
            plan.run()
            ks: list[float] = []
            timed(plan.run, 5, ks)
            forms[label] = {"kernel_ms": float(np.median(ks))}
        plan.set_tune(*tune[:4])
        plan.run()
        ctx.sync()

    ms = float(np.mean(t_batch))
    # replicas: every rank renders its own views; sum pixels, slowest rank's time
    agg = replicas.aggregate(px, ms, dist=dist, device=f"cuda:{local}")
    ms_max = agg["ms"]
    value = agg["gpix_s"]

    peaks = measured_peaks()
    # the dominant kernel's own device time: events recorded inside the graph
    # around the persistent render kernel, read back after every timed step
    k_ms = float(np.mean(t_kernel)) if t_kernel else ms
    l2_gbs = max(ctx.measure_l2_read_gbs() for _ in range(3))
    frame_bytes = 4 * px
    full_s = sum(fs.num_depths(cam_field(v[0], "distance"), wparams) * v[1] for v in views)
    map_bytes = hm.size * 5  # u8 heights + u32 colours, the algorithmic map set
    rl = roofline(frame_bytes, full_s, int(samples), k_ms, peaks["hbm_gbs"], l2_gbs,
                  map_bytes <= L2_BYTES, peaks["source"], capture_figures(name, tune),
                  "render_kernel (persistent, one launch per step)", int(events))

    cpu = cpu1 = None
    if headline and rank == 0 and args.cpu_seconds > 0:
        cpu, cpu1 = cpu_baselines(views, hm, cm, args.cpu_seconds, oracle_params(name))
    plan.close()
    fmap.close()
    del host
    return {
        "metric": METRIC,
        "value": value, "unit": "Gpix/s", "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": ms_max, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded diamond-square maps and cameras)",
        "config": cfg,
        "tune": {"tile_width": tune[0], "lanes_per_column": tune[1], "depth_per_lane": tune[2],
                 "stage": tune[3], "persistent_ctas": tune[4],
                 "autotune_ms": tune_info[1] if tune_info else None},
        "latency_ms": {"p50": float(np.percentile(t_batch, 50)),
                       "p99": float(np.percentile(t_batch, 99))},
        "plain_per_frame": None if not t_plain else {
            "value": px / float(np.mean(t_plain)) / 1e6, "unit": "Gpix/s",
            "ms_per_step": float(np.mean(t_plain)),
            "p50_ms": float(np.percentile(t_plain, 50)),
            "p99_ms": float(np.percentile(t_plain, 99)),
            "launches_per_step": 2 * len(views)},
        "batched_over_plain": None if not t_plain else float(np.mean(t_plain)) / ms,
        "kernel_forms": forms,
        "frames_per_s": len(views) * world / ms_max * 1e3,
        "work": {"depth_samples": samples, "full_depth_samples": full_s,
                 "events_coloured": events},
        "roofline": rl,
        **parity,
        "clocks": clk,
        "e2e": e2e,
        "gpu_launches": gpu_launches,
        "cpu_baseline": cpu,
        "cpu_baseline_one_thread": cpu1,
    }


def extra_summary(d: dict) -> dict:
    """The figures of a shorter workload run beside the headline."""
    keep = ("value", "unit", "steps", "warmup", "ms_per_step", "latency_ms", "frames_per_s",
            "tune", "work", "roofline", "frames_checked_vs_oracle", "differing_pixels",
            "checked_views", "gpu_launches", "clocks", "metric", "config")
    return {k: d[k] for k in keep if k in d}


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
                    help="pin the kernel configuration of the main workload: tile_width,"
                         "lanes_per_column,depth_per_lane,stage (skips the autotuner)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-groups", type=int, default=8,
                    help="view groups of the pipelined render + download in the e2e timing")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip timing the three kernel forms on the main plan")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the shorter workloads run beside the default batch512 line")
    ap.add_argument("--extra-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
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

    import torch
    import futspace_gb300 as fs

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    ctx = fs.Context(local)
    if args.workload == "single1080":
        line = single_leg(fs, ctx, args, rank, world, local, args.steps, args.warmup, dist,
                          with_e2e=not args.no_e2e)
    else:
        line = plan_leg(fs, ctx, args, args.workload, rank, world, local, args.steps,
                        args.warmup, dist, headline=True)
        if args.workload == "batch512" and world == 1 and not args.no_extras:
            ext_args = argparse.Namespace(**{**vars(args), "tune": ""})
            extras = {"single1080": single_leg(fs, ctx, ext_args, rank, world, local,
                                               max(args.extra_steps, 10), 3, None,
                                               with_cpu=False, with_e2e=False)}
            for name in ("walk1080", "large4k"):
                extras[name] = plan_leg(fs, ctx, ext_args, name, rank, world, local,
                                        args.extra_steps, 3, None, headline=False)
            line["extra_workloads"] = {k: extra_summary(v) for k, v in extras.items()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
