"""Randomised parity: seeded random maps (power-of-two, non-power-of-two, with
gap-colour texels), cameras (ordinary, below the terrain, horizon far off the
screen), screen sizes, parameters (filters, gap rules, the mode-B schedule,
smoothing, shading/fog) and kernel configurations, through plain calls and
through plans with the pipelined download; every frame against the oracle."""
import numpy as np
import pytest

from conftest import count_diff

pytestmark = pytest.mark.gpu


def _params(fs, rng):
    kw = {}
    if rng.random() < 0.2:  # the mode-B schedule of tests/futspace.fut
        kw.update(invz_param1=0.005, invz_param2=1.0, magic_number=240.0, gap_rule=1, floor_n=0)
    kw["height_filter"] = int(rng.integers(0, 2))
    kw["color_filter"] = int(rng.integers(0, 2))
    kw.setdefault("gap_rule", int(rng.integers(0, 2)))
    r = rng.random()
    if r < 0.1 and kw["gap_rule"] == 0 and "invz_param2" not in kw:
        kw["smoothing"] = 1
    elif r < 0.2:
        kw.update(effects=int(rng.integers(1, 4)), shade=0.5, fog_start=200.0, fog_end=900.0,
                  fog_color=0xFFA0B0C0)
    return fs.default_params(**kw)


def _camera(fs, rng, hm, h):
    r = rng.random()
    if r < 0.08:  # at or below the terrain
        return fs.Camera(float(rng.uniform(-500, 500)), float(rng.uniform(-500, 500)),
                         float(rng.uniform(-50, 10)), float(rng.uniform(0, 6.3)),
                         float(rng.uniform(-100, h + 100)), float(rng.uniform(50, 1500)), 1.2,
                         0xFF9090E0)
    if r < 0.14:  # the horizon far above or below the screen
        return fs.Camera(float(rng.uniform(0, 300)), float(rng.uniform(0, 300)), 150.0,
                         float(rng.uniform(0, 6.3)), float(rng.choice([1e5, -1e5, h / 2])),
                         float(rng.uniform(50, 1500)), float(rng.uniform(0.5, 2.0)), 0xFF8080D0)
    return fs.gen_cameras(int(rng.integers(0, 1 << 30)), hm, 1, above=(5, 250),
                          distance=(30, 2500), screen_h=h)[0]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_configurations(fs, orc, gpu_ctx, seed):
    rng = np.random.default_rng(seed)
    maps = []
    for k, (size, rough) in enumerate(((256, 0.55), (1024, 0.6), (512, 0.5))):
        hm = fs.gen_heights(900 + k, size, rough)
        cm = fs.gen_colors(950 + k, hm, 12)
        if k == 1:
            cm = cm.copy()
            cm[::7, ::5] = 0
        if k == 2:
            hm, cm = np.ascontiguousarray(hm[:300, :200]), np.ascontiguousarray(cm[:300, :200])
        maps.append((hm, cm, fs.Map(gpu_ctx, hm, cm)))
    table = fs.tune_table()
    frames = 0
    try:
        while frames < 150:
            hm, cm, fmap = maps[int(rng.integers(0, len(maps)))]
            p = _params(fs, rng)
            po = orc.params_from(p)
            if rng.random() < 0.6:
                w, h = int(rng.integers(1, 500)), int(rng.integers(1, 300))
                cam = _camera(fs, rng, hm, h)
                tune = table[int(rng.integers(0, len(table)))] if rng.random() < 0.7 else None
                gpu_ctx.force_tune(tune)
                got = gpu_ctx.render(fmap, cam, w, h, params=p)
                ref = orc.render(cam, po, hm, cm, w, h, threads=0)
                assert count_diff(got, ref) == 0, (seed, frames, tune, w, h, p.smoothing, p.effects)
                frames += 1
            else:
                gpu_ctx.force_tune(None)
                views = []
                for _ in range(int(rng.integers(1, 7))):
                    w, h = int(rng.integers(1, 400)), int(rng.integers(1, 300))
                    views.append((_camera(fs, rng, hm, h), w, h))
                plan = fs.Plan(gpu_ctx, [fmap], views, params=p)
                t = table[int(rng.integers(0, len(table)))]
                try:
                    plan.set_tune(*t)
                except fs.FsError:  # a configuration that does not fit these views
                    pass
                out = np.full(plan.total_pixels, 0xDEADBEEF, np.uint32)
                got = plan.frames(plan.run_download(out, groups=int(rng.integers(1, 17))))
                for (cam, w, h), f in zip(views, got):
                    ref = orc.render(cam, po, hm, cm, w, h, threads=0)
                    assert count_diff(f, ref) == 0, (seed, frames, t, w, h, p.smoothing)
                    frames += 1
                plan.close()
    finally:
        gpu_ctx.force_tune(None)
        for _, _, m in maps:
            m.close()
