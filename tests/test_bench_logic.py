"""The benchmark's own bookkeeping, on the CPU: which committed ncu capture a
line quotes, which frames it checks against the oracle, and the roofline
arithmetic of its `roofline` object (all recomputable from the line)."""
import pytest

import bench


def test_capture_lines_match_the_configuration():
    got = bench.capture_figures("batch512", (64, 2, 4, 0, 1216))
    assert got["capture_tune"] == "64,2,4,0"
    assert got["dram_bytes_per_launch"] > 1e9 and got["l2_read_sectors_per_launch"] > 1e8
    assert bench.capture_figures("batch512", (128, 1, 4, 0, 0))["capture_tune"] == "128,1,4,0"
    # a configuration without a capture, or a workload without a summary: nothing
    assert bench.capture_figures("batch512", (32, 4, 4, 0)) == {}
    assert bench.capture_figures("walk1080", (32, 4, 4, 0)) == {}


def test_check_sample_covers_every_resolution_twice():
    views = [({"distance": float(d)}, w, h)
             for d, (w, h) in zip(range(400, 3000, 100), bench.RESOLUTIONS * 6)]
    idx = bench.check_sample(views)
    per_res = {}
    for i in idx:
        per_res.setdefault(views[i][1:], []).append(i)
    assert set(per_res) == set(bench.RESOLUTIONS)
    assert all(len(v) >= 2 for v in per_res.values())
    # equal distances: the middle and the last view are added
    flat = [({"distance": 3000.0}, 1920, 1080) for _ in range(64)]
    assert bench.check_sample(flat) == [0, 32, 63]


def test_roofline_is_the_slower_term_over_kernel_time():
    frame, s_full, s_eff = 2_815_488_000, 1_223_140_800, 695_554_992
    r = bench.roofline(frame, s_full, s_eff, 3.97, 6788.3, 15000.0, True, "measured", {}, "k")
    t_frame = frame / 6788.3e6
    t_gather = 20 * s_full / 15000.0e6
    assert r["bound"] == "l2" and r["t_roof_ms"] == pytest.approx(max(t_frame, t_gather))
    assert r["frac"] == pytest.approx(r["t_roof_ms"] / 3.97)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert r["effective"]["frac"] == pytest.approx(max(t_frame, 20 * s_eff / 15000.0e6) / 3.97)
    assert r["traffic"] is None and "no committed ncu capture" in r["traffic_source"]
    # maps beyond L2: the gathers go at the HBM copy peak
    r = bench.roofline(frame, s_full, s_eff, 3.97, 6788.3, 15000.0, False, "measured", {}, "k")
    assert r["bound"] == "hbm" and r["peak"] == 6788.3
    # a frame-store bound (few samples)
    r = bench.roofline(frame, 1000, 1000, 1.0, 6788.3, 15000.0, True, "measured", {}, "k")
    assert r["bound"] == "hbm" and r["frac"] == pytest.approx(t_frame / 1.0)


def test_hbm_copy_form_is_kept_as_an_extra():
    r = bench.roofline(100, 10, 5, 1.0, 1000.0, 2000.0, True, "m", {}, "k", events=2)
    assert r["hbm_copy_form"]["bytes"] == 100 + 4 * 5 + 16 * 2
    assert r["hbm_copy_form"]["frac"] == pytest.approx(r["hbm_copy_form"]["achieved"] / 1000.0)
