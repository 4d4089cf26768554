"""GPU parity: every frame the CUDA path renders equals the CPU oracle's, bit
for bit (ARGB u32 output: no tolerance). All calls go through the C ABI."""
import os

import numpy as np
import pytest

from conftest import count_diff

pytestmark = pytest.mark.gpu

FILTERS = [(h, c) for h in (0, 1) for c in (0, 1)]


def _oracle(orc, cam, p, hm, cm, w, h):
    return orc.render(cam, orc.params_from(p), hm, cm, w, h, threads=0)


@pytest.mark.parametrize("hf,cf", FILTERS)
def test_small_frames_all_filters(fs, orc, gpu_ctx, maps256, hf, cf):
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(height_filter=hf, color_filter=cf)
    for cam in fs.gen_cameras(31, hm, 6, above=(20, 80), distance=(150, 500), screen_h=48):
        got = gpu_ctx.render(fmap, cam, 64, 48, params=p)
        assert count_diff(got, _oracle(orc, cam, p, hm, cm, 64, 48)) == 0


def test_config1_frames(fs, orc, gpu_ctx, maps1024):
    """320x240 over a 1024^2 map, D=800 (n=1265), 40 above the local maximum."""
    hm, cm = maps1024
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params()
    for cam in fs.gen_cameras(41, hm, 8, above=(40, 40), distance=(800, 800), screen_h=240):
        got = gpu_ctx.render(fmap, cam, 320, 240)
        assert count_diff(got, _oracle(orc, cam, p, hm, cm, 320, 240)) == 0


def test_every_configuration(fs, orc, gpu_ctx, maps1024):
    """Each compiled kernel configuration, on a TMA-aligned and an odd size."""
    hm, cm = maps1024
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params()
    cams = fs.gen_cameras(51, hm, 2, above=(20, 120), distance=(300, 900), screen_h=120)
    refs = {}
    try:
        for tune in fs.tune_table():
            gpu_ctx.force_tune(tune)
            for i, cam in enumerate(cams):
                for (w, h) in ((160, 120), (157, 97)):
                    key = (i, w, h)
                    if key not in refs:
                        refs[key] = _oracle(orc, cam, p, hm, cm, w, h)
                    got = gpu_ctx.render(fmap, cam, w, h)
                    assert count_diff(got, refs[key]) == 0, (tune, key)
    finally:
        gpu_ctx.force_tune(None)


def test_walk_1080p_4096_map(fs, orc, gpu_ctx):
    """The 64-frame camera walk at 1920x1080 over 4096^2 maps, D=3000, rendered
    as one batch; every frame checked."""
    hm = fs.gen_heights(7, 4096, 0.55)
    cm = fs.gen_colors(8, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    walk = fs.gen_walk(9, hm, 64, step=2.0, yaw=0.02, above=(30, 120), distance=3000.0,
                       screen_h=1080)
    plan = fs.Plan(gpu_ctx, [fmap], [(c, 1920, 1080) for c in walk])
    plan.run()
    frames = plan.frames()
    p = fs.default_params()
    bad = [i for i, (c, f) in enumerate(zip(walk, frames))
           if count_diff(f, _oracle(orc, c, p, hm, cm, 1920, 1080)) != 0]
    assert not bad, f"frames differing from the oracle: {bad}"


def _mixed_views(fs, hm, seed, n):
    sizes = [(320, 240), (640, 480), (257, 131), (128, 96), (203, 64)]
    rng = np.random.default_rng(seed)
    out = []
    for v in range(n):
        w, h = sizes[int(rng.integers(0, len(sizes)))]
        cam = fs.gen_cameras(seed * 100 + v, hm, 1, above=(20, 200), distance=(200, 1200),
                             screen_h=h)[0]
        out.append((cam, w, h))
    return out


def test_batch_plan_all_configurations(fs, orc, gpu_ctx, maps1024):
    hm, cm = maps1024
    fmap = fs.Map(gpu_ctx, hm, cm)
    views = _mixed_views(fs, hm, 61, 24)
    p = fs.default_params()
    refs = [_oracle(orc, c, p, hm, cm, w, h) for c, w, h in views]
    plan = fs.Plan(gpu_ctx, [fmap], views)
    for tune in fs.tune_table():
        plan.set_tune(*tune)
        plan.run()
        frames = plan.frames()
        bad = [i for i, (f, r) in enumerate(zip(frames, refs)) if count_diff(f, r)]
        assert not bad, (tune, bad)
    plan.run_per_view()
    assert all(count_diff(f, r) == 0 for f, r in zip(plan.frames(), refs))
    # pipelined render + download: same frames for any grouping, after a
    # tuning change too (the group lists follow the items)
    buf = fs.PinnedBuffer(plan.total_pixels)
    for groups in (1, 3, 16):
        flat = plan.run_download(buf.array, groups=groups)
        bad = [i for i, (f, r) in enumerate(zip(plan.frames(flat), refs)) if count_diff(f, r)]
        assert not bad, (groups, bad)
        plan.set_tune(*fs.tune_table()[groups % len(fs.tune_table())])


def test_run_download_sky_rows(fs, orc, gpu_ctx, maps256):
    """fs_plan_run_download copies only the rows below each view's all-sky rows
    and writes the sky rows on the host: frames identical to the oracle with
    views whose every row is sky, views with no sky row (camera below the
    terrain), ordinary views, a view split into depth segments, both gap
    rules, every kernel form, pinned and pageable host buffers (stale bytes
    overwritten), and byte counters that add up to the frames."""
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    base = fs.gen_cameras(401, hm, 3, above=(20, 80), distance=(300, 900), screen_h=96)
    views = [(base[0], 128, 96),
             (fs.Camera(60.0, 70.0, -10.0, 0.4, 48.0, 400.0, 1.2, 0xFF9090E0), 96, 64),
             (fs.Camera(80.0, 90.0, 120.0, 1.0, 1.0e5, 400.0, 1.2, 0xFF8080D0), 64, 48),
             (base[1], 257, 131), (base[2], 40, 300)]
    for gap in (0, 1):
        p = fs.default_params(gap_rule=gap)
        refs = [_oracle(orc, c, p, hm, cm, w, h) for c, w, h in views]
        plan = fs.Plan(gpu_ctx, [fmap], views, params=p)
        pinned = fs.PinnedBuffer(plan.total_pixels)
        pageable = np.empty(plan.total_pixels, np.uint32)
        for k, tune in enumerate(fs.tune_table()[::3] + [(8, 64, 8, 2)]):
            plan.set_tune(*tune)
            for groups, buf in ((1, pinned.array), (2, pageable), (5, pinned.array)):
                buf[:] = 0x12345678
                flat = plan.run_download(buf, groups=groups)
                bad = [i for i, (f, r) in enumerate(zip(plan.frames(flat), refs))
                       if count_diff(f, r)]
                assert not bad, (gap, tune, groups, bad)
                copied, filled = plan.download_bytes()
                # every frame's pixels once (the arena's alignment gaps are no frame's)
                assert copied + filled == 4 * sum(w * h for _, w, h in views) + 4 * len(views)
                assert filled >= 4 * 64 * 48  # the all-sky view is written on the host
        pinned.close()
        plan.close()
    # one small view alone: the plan splits its depths into segments
    cam = base[0]
    ref = _oracle(orc, cam, fs.default_params(), hm, cm, 320, 240)
    plan = fs.Plan(gpu_ctx, [fmap], [(cam, 320, 240)])
    for tune in ((64, 2, 4, 0), (128, 1, 4, 0), (32, 8, 4, 0)):
        plan.set_tune(*tune)
        out = np.full(320 * 240, 7, np.uint32)
        assert count_diff(plan.frames(plan.run_download(out, groups=1))[0], ref) == 0, tune
    plan.close()
    fmap.close()


def test_run_download_small_host_team(tmp_path):
    """With OMP_NUM_THREADS=1 the download copies whole frames (no host-written
    sky rows): same frames as the oracle, byte counters of a whole copy."""
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    script = tmp_path / "small_team.py"
    script.write_text(f"""
import sys
sys.path.insert(0, {str(root)!r})
import numpy as np
import futspace_gb300 as fs, oracle
ctx = fs.Context(0)
hm = fs.gen_heights(21, 256, 0.55); cm = fs.gen_colors(22, hm, 12)
fmap = fs.Map(ctx, hm, cm)
cams = fs.gen_cameras(501, hm, 4, above=(20, 80), distance=(300, 900), screen_h=96)
views = [(c, 128, 96) for c in cams]
plan = fs.Plan(ctx, [fmap], views)
out = np.full(plan.total_pixels, 5, np.uint32)
frames = plan.frames(plan.run_download(out, groups=2))
p = oracle.make_params()
bad = sum(int(np.count_nonzero(f != oracle.render(c, p, hm, cm, 128, 96, threads=1)))
          for f, (c, w, h) in zip(frames, views))
copied, filled = plan.download_bytes()
assert bad == 0, bad
assert filled == 0 and copied == 4 * plan.total_pixels, (copied, filled)
print("ok")
""")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr


def test_batch_two_maps_and_camera_update(fs, orc, gpu_ctx, maps1024, maps256):
    (h1, c1), (h2, c2) = maps1024, maps256
    m1, m2 = fs.Map(gpu_ctx, h1, c1), fs.Map(gpu_ctx, h2, c2)
    views = [(c, w, h, i % 2) for i, (c, w, h) in enumerate(_mixed_views(fs, h1, 71, 10))]
    plan = fs.Plan(gpu_ctx, [m1, m2], views)
    p = fs.default_params()
    for step in range(2):
        plan.run()
        frames = plan.frames()
        for (c, w, h, mi), f in zip(views, frames):
            hm, cm = (h1, c1) if mi == 0 else (h2, c2)
            assert count_diff(f, _oracle(orc, c, p, hm, cm, w, h)) == 0
        # move every camera; draw distances shrink so the depth tables still fit
        new = []
        for c, w, h, mi in views:
            c2_ = fs.Camera(*c.as_tuple())
            c2_.x += 3.5
            c2_.angle += 0.25
            c2_.distance *= 0.9
            new.append((c2_, w, h, mi))
        plan.set_cameras([v[0] for v in new])
        views = new


@pytest.mark.parametrize("hf,cf", FILTERS)
@pytest.mark.parametrize("gap", [0, 1])
def test_adversarial_inputs(fs, orc, gpu_ctx, maps256, hf, cf, gap):
    """Zero-colour and sky-colour texels, integral and negative coordinates,
    cameras below or exactly at the terrain (z = 0 hazards), both gap rules."""
    hm, cm = maps256
    cm = cm.copy()
    cm[::3, ::2] = 0
    cm[1::5, 1::3] = 0xFF9090E0
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(height_filter=hf, color_filter=cf, gap_rule=gap)
    at = orc.lib().fso_height_bilinear(hm.ctypes.data, 256, 256, 64.5, 64.25)
    cams = [dict(x=100.0, y=100.0, height=300.0, angle=0.0, horizon=24.0, distance=200.0),
            dict(x=-37.0, y=-300.0, height=120.0, angle=1.5707964, horizon=30.0,
                 distance=400.0),
            dict(x=64.5, y=64.25, height=-10.0, angle=0.3, horizon=24.0, distance=150.0),
            dict(x=64.5, y=64.25, height=at, angle=0.3, horizon=24.0, distance=150.0)]
    for c in cams:
        cam = fs.Camera(c["x"], c["y"], c["height"], c["angle"], c["horizon"], c["distance"],
                        1.2, 0xFF9090E0)
        got = gpu_ctx.render(fmap, cam, 61, 47, params=p)
        assert count_diff(got, _oracle(orc, cam, p, hm, cm, 61, 47)) == 0


def test_mode_b_and_custom_scale(fs, orc, gpu_ctx, maps256):
    """tests/futspace.fut parameters: nearest, z0=1, d=0.005, scale 240, gap=sky."""
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(invz_param1=0.005, invz_param2=1.0, magic_number=240.0,
                          height_filter=0, color_filter=0, gap_rule=1, floor_n=0)
    cam = fs.Camera(128.0, 200.0, 78.0, 0.0, 100.0, 800.0, 1.0, 0xFF9090E0)
    got = gpu_ctx.render(fmap, cam, 800, 400, params=p)
    assert count_diff(got, _oracle(orc, cam, p, hm, cm, 800, 400)) == 0


def test_non_power_of_two_map_and_i32_heights(fs, orc, gpu_ctx):
    hm = fs.gen_heights(3, 512, 0.6)[:300, :200].copy()
    cm = fs.gen_colors(4, hm, 12)
    # i32 heights with junk above bit 7: update_map keeps `elem & 0xFF`
    hi = hm.astype(np.int32) | (np.int32(0x5A) << 8)
    fmap = fs.Map(gpu_ctx, hi, cm)
    p = fs.default_params()
    for cam in fs.gen_cameras(9, hm, 3, above=(30, 60), distance=(300, 700), screen_h=90):
        got = gpu_ctx.render(fmap, cam, 120, 90)
        assert count_diff(got, _oracle(orc, cam, p, hm, cm, 120, 90)) == 0


@pytest.mark.parametrize("hf,cf", FILTERS)
def test_non_power_of_two_map_every_configuration(fs, orc, gpu_ctx, hf, cf):
    """Every compiled configuration (direct painting, staged tiles, cooperative
    tiles) on a 300x200 map, whose height and colour wraps are the floored
    modulo rather than a mask, for both filters, plus the smoothing and
    shading/fog modes."""
    hm = fs.gen_heights(13, 512, 0.6)[:300, :200].copy()
    cm = fs.gen_colors(14, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(height_filter=hf, color_filter=cf)
    cams = fs.gen_cameras(15, hm, 2, above=(20, 80), distance=(250, 900), screen_h=61)
    cams.append(fs.Camera(-450.25, 910.5, 140.0, 2.4, 30.0, 600.0, 1.1, 0xFF9090E0))
    sizes = ((97, 61), (64, 130))
    refs = {(i, w, h): _oracle(orc, c, p, hm, cm, w, h)
            for i, c in enumerate(cams) for w, h in sizes}
    try:
        for tune in fs.tune_table():
            gpu_ctx.force_tune(tune)
            for (i, w, h), ref in refs.items():
                got = gpu_ctx.render(fmap, cams[i], w, h, params=p)
                assert count_diff(got, ref) == 0, (tune, i, w, h)
    finally:
        gpu_ctx.force_tune(None)
    for extra in (dict(smoothing=1),
                  dict(effects=3, shade=0.5, fog_start=50.0, fog_end=600.0,
                       fog_color=0xFFA0B0C0)):
        pm = fs.default_params(height_filter=hf, color_filter=cf, **extra)
        for c in cams:
            assert count_diff(gpu_ctx.render(fmap, c, 97, 61, params=pm),
                              _oracle(orc, c, pm, hm, cm, 97, 61)) == 0, extra


def test_chunk_skip_is_exact_and_saves_work(fs, orc, gpu_ctx):
    """The max-pyramid chunk skip changes no pixel and evaluates fewer samples."""
    hm = fs.gen_heights(17, 1024, 0.55)
    cm = fs.gen_colors(18, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    views = _mixed_views(fs, hm, 81, 12)
    p = fs.default_params()
    counts = {}
    for skip in (0, 1):
        gpu_ctx.set_option("skip", skip)
        try:
            for tune in fs.tune_table():
                gpu_ctx.force_tune(tune)
                gpu_ctx.stats(True)
                for c, w, h in views:
                    got = gpu_ctx.render(fmap, c, w, h)
                    assert count_diff(got, _oracle(orc, c, p, hm, cm, w, h)) == 0, (skip, tune)
                counts[(skip, tune)] = gpu_ctx.stats(True)
        finally:
            gpu_ctx.force_tune(None)
            gpu_ctx.set_option("skip", 1)
    for tune in fs.tune_table():
        s_off, e_off = counts[(0, tune)]
        s_on, e_on = counts[(1, tune)]
        assert e_on == e_off          # the same occlusion events are coloured
        assert s_on < s_off           # fewer depth samples are evaluated


@pytest.mark.parametrize("effects", [1, 2, 3])
def test_effects_epilogue(fs, orc, gpu_ctx, maps1024, effects):
    """Depth shading / fog fused into the colour path: bit-exact vs the oracle,
    for single frames (every configuration) and a batch plan."""
    hm, cm = maps1024
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(effects=effects, shade=0.5, fog_start=100.0, fog_end=900.0,
                          fog_color=0xFFA0B0C0)
    views = _mixed_views(fs, hm, 101 + effects, 6)
    refs = [_oracle(orc, c, p, hm, cm, w, h) for c, w, h in views]
    try:
        for tune in fs.tune_table():
            gpu_ctx.force_tune(tune)
            for (c, w, h), r in zip(views[:2], refs[:2]):
                assert count_diff(gpu_ctx.render(fmap, c, w, h, params=p), r) == 0, tune
    finally:
        gpu_ctx.force_tune(None)
    plan = fs.Plan(gpu_ctx, [fmap], views, params=p)
    plan.run()
    assert all(count_diff(f, r) == 0 for f, r in zip(plan.frames(), refs))
    with pytest.raises(fs.FsError):
        gpu_ctx.render(fmap, views[0][0], 64, 48,
                       params=fs.default_params(effects=2, fog_start=5.0, fog_end=5.0))


def test_large_map_4k_with_effects(fs, orc, gpu_ctx):
    """3840x2160 frames, D=6000 (n=3464), over a 16384^2 map (beyond L2), with the
    depth shading + fog epilogue: bit-exact vs the oracle."""
    hm = fs.gen_heights(107, 16384, 0.6)
    cm = fs.gen_colors(108, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(effects=3, shade=0.5, fog_start=1500.0, fog_end=6000.0,
                          fog_color=0xFFA0B0C0)
    cams = fs.gen_cameras(109, hm, 2, above=(30, 150), distance=(6000, 6000), screen_h=2160)
    plan = fs.Plan(gpu_ctx, [fmap], [(c, 3840, 2160) for c in cams], params=p)
    plan.run()
    for c, f in zip(cams, plan.frames()):
        assert count_diff(f, _oracle(orc, c, p, hm, cm, 3840, 2160)) == 0
    fmap.close()


@pytest.mark.parametrize("hf,cf", FILTERS)
def test_smoothing_branch(fs, orc, gpu_ctx, maps256, hf, cf):
    """`#on` smoothing: single frames, a batch plan and near-field cameras that
    blend many rows; bit-exact vs the oracle."""
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(height_filter=hf, color_filter=cf, smoothing=1)
    views = _mixed_views(fs, hm, 111 + hf + 2 * cf, 6)
    near = fs.Camera(100.5, 80.25, float(hm[80, 100]) + 3.0, 0.7, 20.0, 60.0, 1.2, 0xFF9090E0)
    views.append((near, 64, 40))
    for c, w, h in views:
        assert count_diff(gpu_ctx.render(fmap, c, w, h, params=p),
                          _oracle(orc, c, p, hm, cm, w, h)) == 0
    plan = fs.Plan(gpu_ctx, [fmap], views, params=p)
    plan.run()
    for (c, w, h), f in zip(views, plan.frames()):
        assert count_diff(f, _oracle(orc, c, p, hm, cm, w, h)) == 0
    with pytest.raises(fs.FsError):
        gpu_ctx.render(fmap, views[0][0], 64, 48,
                       params=fs.default_params(smoothing=1, gap_rule=1))


@pytest.mark.parametrize("hf,cf", [(1, 1), (0, 1)])
def test_depth_segments_exact(fs, orc, gpu_ctx, maps1024, hf, cf):
    """Columns split into depth segments (segment-minimum pass, render pass from
    the prefix minimum, gap-fill pass) give the same frames as unsplit columns,
    for single frames and plans, with zero texels forcing the gap fill."""
    hm, cm = maps1024
    cm = cm.copy()
    cm[::5, ::3] = 0          # gap colour (gap rule 0) in the map
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(height_filter=hf, color_filter=cf)
    views = _mixed_views(fs, hm, 131 + hf + 2 * cf, 6)
    refs = [_oracle(orc, c, p, hm, cm, w, h) for c, w, h in views]
    direct = [t for t in fs.tune_table() if t[3] == 0]
    for tune in direct[::3]:
        gpu_ctx.force_tune(tune)
        splits = 0
        for (c, w, h), r in zip(views, refs):
            l0 = gpu_ctx.launches
            got = gpu_ctx.render(fmap, c, w, h, params=p)
            assert count_diff(got, r) == 0, (tune, w, h)
            splits += gpu_ctx.launches - l0 > 2
            gpu_ctx.set_option("split", 0)
            l0 = gpu_ctx.launches
            assert count_diff(gpu_ctx.render(fmap, c, w, h, params=p), r) == 0
            assert gpu_ctx.launches - l0 == 2
            gpu_ctx.set_option("split", 1)
        assert splits > 0, tune  # frames this small have too few strips: they split
    gpu_ctx.force_tune(None)
    # a plan of few views splits too; shorter draw distances later leave
    # trailing segments empty
    plan = fs.Plan(gpu_ctx, [fmap], views, params=p)
    for tune in direct[::4]:
        plan.set_tune(*tune)
        plan.run()
        assert all(count_diff(f, r) == 0 for f, r in zip(plan.frames(), refs)), tune
    cams = []
    for c, w, h in views:
        d = fs.Camera(*c.as_tuple())
        d.distance = c.distance * 0.5
        cams.append(d)
    plan.set_cameras(cams)
    plan.run()
    for i, ((c, w, h), f) in enumerate(zip(views, plan.frames())):
        assert count_diff(f, _oracle(orc, cams[i], p, hm, cm, w, h)) == 0
    buf = fs.PinnedBuffer(plan.total_pixels)
    flat = plan.run_download(buf.array, groups=3)
    for i, ((c, w, h), f) in enumerate(zip(views, plan.frames(flat))):
        assert count_diff(f, _oracle(orc, cams[i], p, hm, cm, w, h)) == 0


def test_degenerate_screen_sizes(fs, orc, gpu_ctx, maps256):
    """One-pixel and one-row/one-column screens, tall thin and short wide ones,
    with the default (possibly split) configuration and every direct-paint
    configuration."""
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params()
    cam = fs.gen_cameras(151, hm, 1, above=(30, 30), distance=(600, 600), screen_h=64)[0]
    sizes = [(1, 1), (1, 9), (9, 1), (3, 300), (300, 3), (33, 17), (65, 2)]
    for tune in [None] + [t for t in fs.tune_table() if t[3] == 0][::4]:
        gpu_ctx.force_tune(tune)
        for w, h in sizes:
            got = gpu_ctx.render(fmap, cam, w, h, params=p)
            assert got.shape == (h, w)
            assert count_diff(got, _oracle(orc, cam, p, hm, cm, w, h)) == 0, (tune, w, h)
    gpu_ctx.force_tune(None)
    plan = fs.Plan(gpu_ctx, [fmap], [(cam, w, h) for w, h in sizes])
    plan.run()
    for (w, h), f in zip(sizes, plan.frames()):
        assert count_diff(f, _oracle(orc, cam, p, hm, cm, w, h)) == 0, (w, h)


@pytest.mark.parametrize("hf,cf", FILTERS)
def test_cooperative_tile_exact(fs, orc, gpu_ctx, maps256, hf, cf):
    """The cooperative tile form (stage 2: a CTA marches all depth blocks of its
    columns at once, min-scan across threads) on adversarial cameras (below and
    at the terrain: every column reaches row 0 early), a non-power-of-two map,
    degenerate and odd screen sizes, both gap rules and the mode-B schedule."""
    hm, cm = maps256
    cm = cm.copy()
    cm[::3, ::2] = 0
    fmap = fs.Map(gpu_ctx, hm, cm)
    hn = fs.gen_heights(3, 512, 0.6)[:300, :200].copy()
    cn = fs.gen_colors(4, hn, 12)
    fmap_n = fs.Map(gpu_ctx, hn, cn)
    at = orc.lib().fso_height_bilinear(hm.ctypes.data, 256, 256, 64.5, 64.25)
    cams = [fs.Camera(100.0, 100.0, 300.0, 0.0, 24.0, 200.0, 1.2, 0xFF9090E0),
            fs.Camera(-37.0, -300.0, 120.0, 1.5707964, 30.0, 400.0, 1.2, 0xFF9090E0),
            fs.Camera(64.5, 64.25, -10.0, 0.3, 24.0, 150.0, 1.2, 0xFF9090E0),
            fs.Camera(64.5, 64.25, at, 0.3, 24.0, 150.0, 1.2, 0xFF9090E0)]
    cams += fs.gen_cameras(161, hm, 2, above=(20, 90), distance=(400, 1500), screen_h=96)
    coop = [t for t in fs.tune_table() if t[3] == 2]
    assert coop
    try:
        for tune in coop:
            gpu_ctx.force_tune(tune)
            for gap in (0, 1):
                p = fs.default_params(height_filter=hf, color_filter=cf, gap_rule=gap)
                for cam in cams:
                    for w, h in ((61, 47), (128, 96), (1, 1), (3, 300), (300, 3)):
                        got = gpu_ctx.render(fmap, cam, w, h, params=p)
                        ref = _oracle(orc, cam, p, hm, cm, w, h)
                        assert count_diff(got, ref) == 0, (tune, gap, w, h)
            p = fs.default_params(height_filter=hf, color_filter=cf)
            for cam in fs.gen_cameras(9, hn, 2, above=(30, 60), distance=(300, 700),
                                      screen_h=90):
                got = gpu_ctx.render(fmap_n, cam, 120, 90, params=p)
                assert count_diff(got, _oracle(orc, cam, p, hn, cn, 120, 90)) == 0, tune
            pb = fs.default_params(invz_param1=0.005, invz_param2=1.0, magic_number=240.0,
                                   height_filter=hf, color_filter=cf, gap_rule=1, floor_n=0)
            cam = fs.Camera(128.0, 200.0, 78.0, 0.0, 100.0, 800.0, 1.0, 0xFF9090E0)
            got = gpu_ctx.render(fmap, cam, 800, 400, params=pb)
            assert count_diff(got, _oracle(orc, cam, pb, hm, cm, 800, 400)) == 0, tune
    finally:
        gpu_ctx.force_tune(None)


def test_cooperative_tile_1080p_frame(fs, orc, gpu_ctx):
    """A 1920x1080 frame over 4096^2 maps at D=3000 (2449 depths: several depth
    blocks per tile) through every cooperative configuration, alone and in a
    batch plan."""
    hm = fs.gen_heights(7, 4096, 0.55)
    cm = fs.gen_colors(8, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    walk = fs.gen_walk(9, hm, 3, step=2.0, yaw=0.02, above=(30, 120), distance=3000.0,
                       screen_h=1080)
    p = fs.default_params()
    refs = [_oracle(orc, c, p, hm, cm, 1920, 1080) for c in walk]
    coop = [t for t in fs.tune_table() if t[3] == 2]
    try:
        for tune in coop:
            gpu_ctx.force_tune(tune)
            for c, ref in zip(walk, refs):
                assert count_diff(gpu_ctx.render(fmap, c, 1920, 1080), ref) == 0, tune
    finally:
        gpu_ctx.force_tune(None)
    plan = fs.Plan(gpu_ctx, [fmap], [(c, 1920, 1080) for c in walk])
    for tune in coop:
        plan.set_tune(*tune)
        plan.run()
        bad = [i for i, (f, r) in enumerate(zip(plan.frames(), refs)) if count_diff(f, r)]
        assert not bad, (tune, bad)


def test_cooperative_tile_block_boundaries(fs, orc, gpu_ctx, maps256):
    """Depth counts at the cooperative tile's block boundaries (one block short
    of full, exactly one or two 512-depth blocks, one depth past them, 256-depth
    blocks likewise), plain and as one plan whose persistent CTAs take several
    tiles of different views in turn."""
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params()
    views = []
    for k, n in enumerate((300, 256, 257, 511, 512, 513, 1024, 1025)):
        D = 0.001 * n * n / 2.0  # the middle of the distances that give n depths
        assert fs.num_depths(D) == n
        cam = fs.gen_cameras(300 + k, hm, 1, above=(10, 40), distance=(D, D), screen_h=72)[0]
        views.append((cam, 88 if k % 2 else 96, 72))
    refs = [_oracle(orc, c, p, hm, cm, w, h) for c, w, h in views]
    coop = [t for t in fs.tune_table() if t[3] == 2]
    try:
        for tune in coop:
            gpu_ctx.force_tune(tune)
            for (c, w, h), ref in zip(views, refs):
                assert count_diff(gpu_ctx.render(fmap, c, w, h), ref) == 0, (tune, c.distance)
    finally:
        gpu_ctx.force_tune(None)
    plan = fs.Plan(gpu_ctx, [fmap], views)
    for tune in coop:
        plan.set_tune(*tune[:3], 2, 8)  # 8 persistent CTAs: several tiles each
        plan.run()
        bad = [i for i, (f, r) in enumerate(zip(plan.frames(), refs)) if count_diff(f, r)]
        assert not bad, (tune, bad)
    plan.close()
    fmap.close()


def test_plain_call_kernel_timer(fs, gpu_ctx, maps256):
    """Option "time": events around the render kernels of a plain call; no pixel
    changes, and reading the timer before any timed call is a state error."""
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    cam = fs.gen_cameras(171, hm, 1, above=(30, 30), distance=(500, 500), screen_h=96)[0]
    ref = gpu_ctx.render(fmap, cam, 128, 96)
    with pytest.raises(fs.FsError) as ei:
        gpu_ctx.kernel_ms()
    assert ei.value.code == 6
    gpu_ctx.set_option("time", 1)
    try:
        got = gpu_ctx.render(fmap, cam, 128, 96)
        ms = gpu_ctx.kernel_ms()
    finally:
        gpu_ctx.set_option("time", 0)
    assert count_diff(got, ref) == 0
    assert 0.0 < ms < 1000.0


def test_l2_read_probe(gpu_ctx):
    """The roofline's L2 read bandwidth probe returns a finite positive rate."""
    gbs = gpu_ctx.measure_l2_read_gbs(16 << 20, 8)
    assert 100.0 < gbs < 1.0e6


def test_cooperative_tile_limits(fs, orc, gpu_ctx, maps256):
    """The cooperative tile's event list holds a whole tile's events (at most
    TW x H): a 3000-row frame through the 4-column tile; and views beyond its
    32-bit event entries (more than 2^17 depths) fall back to another kernel
    form, alone and in a plan, with the same pixels."""
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params()
    tall = fs.Camera(100.0, 100.0, 180.0, 0.7, 2900.0, 900.0, 1.2, 0xFF9090E0)
    gpu_ctx.force_tune((4, 64, 4, 2))
    try:
        got = gpu_ctx.render(fmap, tall, 40, 3000)
        assert count_diff(got, _oracle(orc, tall, p, hm, cm, 40, 3000)) == 0
        # 131,073+ depths: D = 8.6 million map units at the default depth step
        D = 131075.0 ** 2 / 2000.0
        assert fs.num_depths(D) > 1 << 17
        far = fs.Camera(60.0, 70.0, 300.0, 0.4, 24.0, D, 1.2, 0xFF9090E0)
        got = gpu_ctx.render(fmap, far, 48, 48)
        assert count_diff(got, _oracle(orc, far, p, hm, cm, 48, 48)) == 0
    finally:
        gpu_ctx.force_tune(None)
    plan = fs.Plan(gpu_ctx, [fmap], [(far, 48, 48)])
    with pytest.raises(fs.FsError):
        plan.set_tune(8, 64, 8, 2)
    plan.run()
    assert count_diff(plan.frames()[0], _oracle(orc, far, p, hm, cm, 48, 48)) == 0
    plan.close()
    fmap.close()
