"""The CPU oracle: known answers, and the C restatement against the independent
numpy restatement on adversarial small cases (bit-exact)."""
import numpy as np
import pytest

from conftest import count_diff


# depth-sample counts of get_zs (fut/voxel_renderer.fut:28-34) with the
# reference defaults d=0.001, z0=0, and of tests/futspace.fut:47-53 (d=0.005, z0=1)
KAT_N = {400.0: 894, 800.0: 1265, 1000.0: 1414, 1600.0: 1789, 2000.0: 2000, 3000.0: 2449,
         6000.0: 3464}


@pytest.mark.parametrize("D,n", sorted(KAT_N.items()))
def test_depth_count_kat(orc, D, n):
    assert orc.lib().fso_num_depths(D, 0.001, 0.0, 1) == n


def test_depth_count_mode_b(orc):
    assert orc.lib().fso_num_depths(800.0, 0.005, 1.0, 0) == 400


def test_zs_series(orc):
    from oracle import literal
    zs = orc.get_zs(800.0)
    assert zs[0] == 0.0  # z_1 = 0: inv_z is +inf for the first slice
    np.testing.assert_array_equal(zs, literal.get_zs(800.0, 0.001, 0.0))
    zb = orc.get_zs(800.0, 0.005, 1.0, 0)
    assert zb[0] == 1.0 and zb.size == 400
    np.testing.assert_array_equal(zb, literal.get_zs(800.0, 0.005, 1.0, 0))
    assert orc.lib().fso_num_depths(-5.0, 0.001, 0.0, 1) < 1  # empty range


def test_f2i_saturates(orc):
    L = orc.lib()
    assert L.fso_f2i(float("inf")) == 2**31 - 1
    assert L.fso_f2i(float("-inf")) == -(2**31)
    assert L.fso_f2i(float("nan")) == 0
    assert L.fso_f2i(-1.5) == -1 and L.fso_f2i(2.9) == 2
    assert L.fso_mod(-1, 1024) == 1023 and L.fso_mod(-1024, 1024) == 0


def test_mix_rules(orc):
    from oracle import literal
    L = orc.lib()
    for c in (0xFF123456, 0x00000000, 0xFFFFFFFF, 0x80FF0001):
        assert L.fso_mix(1.0, c, 0.0, 0xDEADBEEF) == c  # full weight returns the colour
        assert L.fso_mix(0.0, c, 0.0, c) == 0           # 0/0 weights: NaN channels -> 0
    rng = np.random.default_rng(3)
    w1 = rng.random(2000).astype(np.float32)
    w2 = rng.random(2000).astype(np.float32)
    c1 = rng.integers(0, 2**32, 2000, dtype=np.uint64).astype(np.uint32)
    c2 = rng.integers(0, 2**32, 2000, dtype=np.uint64).astype(np.uint32)
    got = np.array([L.fso_mix(float(a), int(b), float(c), int(d)) for a, b, c, d in
                    zip(w1, c1, w2, c2)], np.uint32)
    np.testing.assert_array_equal(got, literal.mix(w1, c1, w2, c2))


def _case(fs, orc, hm, cm, cam, W, H, **kw):
    from oracle import literal
    p = orc.make_params(**kw)
    a = orc.render(cam, p, hm, cm, W, H)
    b = literal.render(cam, hm, cm, W, H, d=p.d, z0=p.z0, scale=p.scale,
                       height_filter=p.height_filter, color_filter=p.color_filter,
                       gap_rule=p.gap_rule, floor_n=p.floor_n, effects=p.effects, shade=p.shade,
                       fog_start=p.fog_start, fog_end=p.fog_end, fog_color=p.fog_color,
                       smoothing=p.smoothing)
    assert count_diff(a, b) == 0
    return a


@pytest.mark.parametrize("hf,cf", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("gap", [0, 1])
def test_restatements_agree(fs, orc, maps256, hf, cf, gap):
    hm, cm = maps256
    for cam in fs.gen_cameras(5 + hf + 2 * cf, hm, 3, above=(10, 90), distance=(100, 400),
                              screen_h=40):
        _case(fs, orc, hm, cm, cam, 56, 40, height_filter=hf, color_filter=cf, gap_rule=gap)


def test_mode_b_parameters(fs, orc, maps256):
    """tests/futspace.fut: nearest samplers, z0=1, d=0.005, scale 240, gap = sky."""
    hm, cm = maps256
    cam = dict(x=128.0, y=200.0, height=78.0, angle=0.0, horizon=20.0, distance=300.0, fov=1.0,
               sky_color=0xFF9090E0)
    _case(fs, orc, hm, cm, cam, 80, 40, d=0.005, z0=1.0, scale=240.0, height_filter=0,
          color_filter=0, gap_rule=1, floor_n=0)


def test_integral_and_negative_coordinates(fs, orc, maps256):
    """Integral sample coordinates zero the bilinear weights; negative ones wrap."""
    hm, cm = maps256
    for x, y, ang in ((100.0, 100.0, 0.0), (-37.0, -300.0, 1.5707964), (0.0, 0.0, 3.1415927)):
        cam = dict(x=x, y=y, height=300.0, angle=ang, horizon=24.0, distance=200.0, fov=1.0,
                   sky_color=0xFF9090E0)
        _case(fs, orc, hm, cm, cam, 64, 48)
        _case(fs, orc, hm, cm, cam, 64, 48, d=0.005, z0=1.0, scale=240.0)


def test_camera_at_or_below_terrain(fs, orc, maps256):
    """z_1 = 0 gives inv_z = +inf: a camera below the terrain projects the first
    slice to -inf (row 0) and one exactly at the terrain height to NaN (row 0);
    both collapse every column to one colour, in both restatements."""
    hm, cm = maps256
    x, y = 64.5, 64.25
    at = orc.lib().fso_height_bilinear(hm.ctypes.data, 256, 256, x, y)
    assert at > 0.0
    for height in (-10.0, at):
        cam = dict(x=x, y=y, height=height, angle=0.3, horizon=24.0, distance=150.0,
                   fov=1.2, sky_color=0xFF9090E0)
        f = _case(fs, orc, hm, cm, cam, 40, 30)
        assert np.all(f == f[0:1, :])


def test_zero_and_sky_texels(fs, orc, maps256):
    hm, cm = maps256
    cm = cm.copy()
    cm[::3, ::2] = 0
    cm[1::5, 1::3] = 0xFF9090E0
    for cam in fs.gen_cameras(77, hm, 3, above=(20, 60), distance=(200, 300), screen_h=48):
        for gap in (0, 1):
            for cf in (0, 1):
                _case(fs, orc, hm, cm, cam, 64, 48, color_filter=cf, gap_rule=gap)


def test_non_power_of_two_map(fs, orc):
    hm = fs.gen_heights(3, 256, 0.6)[:200, :150].copy()
    cm = fs.gen_colors(4, hm, 12)
    for cam in fs.gen_cameras(9, hm, 3, above=(30, 60), distance=(300, 500), screen_h=36):
        _case(fs, orc, hm, cm, cam, 48, 36)


def test_multithreaded_oracle_matches(fs, orc, maps1024):
    hm, cm = maps1024
    cam = fs.gen_cameras(13, hm, 1, above=(40, 40), distance=(800, 800), screen_h=240)[0]
    a = orc.render(cam, orc.make_params(), hm, cm, 320, 240)
    b = orc.render(cam, orc.make_params(), hm, cm, 320, 240, threads=4)
    assert count_diff(a, b) == 0


def test_shadowmap_restatement(fs, orc):
    """generate_shadowmap_accumulated (fut/effects.fut:108-125) vs a direct
    evaluation of the same expressions in numpy at a few texels."""
    from oracle import literal
    hm = fs.gen_heights(31, 256, 0.55)
    cm = fs.gen_colors(32, hm, 12)
    sun = np.array([0.6, 0.08, 0.4], np.float32)
    out = orc.shadowmap(hm, cm, sun, threads=4)
    f = np.float32
    for (y, x) in ((0, 0), (17, 300), (1023, 5), (500, 500)):
        fx, fy = f(x), f(y)
        height = f(hm[y % 256, x % 256])
        count = 0
        for dist in range(1, 256):
            t = f(dist) * f(4)
            hx, hy = f(fx + t * sun[0]), f(fy + t * sun[2])
            hs = f(hm[int(literal.f2i(hy)) % 256, int(literal.f2i(hx)) % 256])
            if f(f(height + t * sun[1]) - hs) < f(-0.5):
                count += 1
        want = literal.mix(f(4) * f(count), np.uint32(0xFF000000), f(1), cm[y % 256, x % 256])
        assert int(out[y, x]) == int(want)


@pytest.mark.parametrize("effects", [1, 2, 3])
def test_effects_restatements_agree(fs, orc, maps256, effects):
    """The optional shading/fog epilogue (not part of the reference path)."""
    hm, cm = maps256
    for cam in fs.gen_cameras(91, hm, 3, above=(20, 90), distance=(200, 500), screen_h=40):
        _case(fs, orc, hm, cm, cam, 56, 40, effects=effects, shade=0.6, fog_start=50.0,
              fog_end=float(cam.distance) * 0.8, fog_color=0xFFB0B8C8)


@pytest.mark.parametrize("hf,cf", [(1, 1), (0, 0), (1, 0)])
def test_smoothing_restatements_agree(fs, orc, maps256, hf, cf):
    """The `#on` smoothing branch (fut/voxel_renderer.fut:175-213)."""
    hm, cm = maps256
    for cam in fs.gen_cameras(93 + hf + 2 * cf, hm, 4, above=(10, 90), distance=(100, 400),
                              screen_h=40):
        on = _case(fs, orc, hm, cm, cam, 56, 40, height_filter=hf, color_filter=cf,
                   smoothing=1)
        assert on.shape == (40, 56)
    # near-field cameras low over the terrain blend many rows
    cam = dict(x=100.5, y=80.25, height=float(hm[80, 100]) + 3.0, angle=0.7, horizon=20.0,
               distance=60.0, fov=1.2, sky_color=0xFF9090E0)
    on = _case(fs, orc, hm, cm, cam, 64, 40, smoothing=1)
    off = _case(fs, orc, hm, cm, cam, 64, 40)
    assert count_diff(on, off) > 0
