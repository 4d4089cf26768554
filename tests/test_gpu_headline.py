"""Bit-exactness on the benchmark's headline configuration and on the
reference's own terrain.

* The batch512 plan itself: 512 views over the 4096^2 map pair, resolutions
  320x240..2560x1440, D in [400, 3000], built exactly as bench.py builds it and
  rendered by one persistent launch; per resolution the views with the largest
  and the smallest draw distance are diffed against the oracle (0 differing
  pixels), under the default tuning and under the batch autotuner's usual pick.
* The reference's map images (data/converted-maps/C1W.png + D1.png, 1024^2, and
  D1_4k.png, 4096^2, with a seeded colour map because its colour partner is not
  in the reference tree), every filter pair, against the oracle. Heights are
  the low byte of each height-image word (fut/interactive.fut:189). These read
  the reference checkout named by FUTSPACE_REFERENCE_DIR and skip without it.
"""
import numpy as np
import pytest

from conftest import count_diff, reference_dir

pytestmark = pytest.mark.gpu


def _bench():
    import bench
    return bench


@pytest.mark.parametrize("tune", [None, (64, 2, 4, 0, 0), (8, 64, 8, 2, 0)])
def test_batch512_plan_sampled_frames(fs, orc, gpu_ctx, tune):
    b = _bench()
    hm, cm, views, _ = b.make_workload(b.ProductGen(fs), "batch512", 0)
    fmap = fs.Map(gpu_ctx, hm, cm)
    plan = fs.Plan(gpu_ctx, [fmap], views)
    if tune:
        plan.set_tune(*tune)
    plan.run()
    flat = plan.download()
    idx = b.check_sample(views)
    assert len(idx) == 10
    # the two 2560x1440 views include the one with the largest draw distance
    big = [i for i in idx if views[i][1] == 2560]
    assert max(views[i][0].distance for i in big) == max(
        v[0].distance for v in views if v[1] == 2560)
    p = orc.make_params()
    for i in idx:
        cam, w, h = views[i]
        o = plan.frame_offset(i)
        got = flat[o:o + w * h].reshape(h, w)
        want = orc.render(cam, p, hm, cm, w, h, threads=0)
        assert count_diff(got, want) == 0, (i, w, h, cam.distance)
    plan.close()
    fmap.close()


def _ref_maps():
    ref = reference_dir()
    if ref is None or not (ref / "data" / "converted-maps" / "D1.png").exists():
        pytest.skip("reference map images not present (set FUTSPACE_REFERENCE_DIR)")
    return ref / "data" / "converted-maps"


@pytest.mark.parametrize("hf,cf", [(1, 1), (1, 0), (0, 1), (0, 0)])
def test_reference_terrain_1024(fs, orc, gpu_ctx, hf, cf):
    d = _ref_maps()
    fmap = fs.Map.from_png(gpu_ctx, d / "C1W.png", d / "D1.png")
    hm = (fs.png_read(d / "D1.png") & 0xFF).astype(np.uint8)
    cm = fs.png_read(d / "C1W.png")
    p = fs.default_params(height_filter=hf, color_filter=cf)
    op = orc.params_from(p)
    for cam, w, h in ([(c, 640, 480) for c in fs.gen_cameras(31, hm, 2, above=(10, 80),
                                                              distance=(800, 1600), screen_h=480)]
                      + [(c, 1920, 1080) for c in fs.gen_cameras(32, hm, 1, above=(20, 120),
                                                                  distance=(3000, 3000),
                                                                  screen_h=1080)]):
        got = gpu_ctx.render(fmap, cam, w, h, params=p)
        want = orc.render(cam, op, hm, cm, w, h, threads=0)
        assert count_diff(got, want) == 0, (w, h, cam.as_tuple())
    fmap.close()


@pytest.mark.parametrize("hf,cf", [(1, 1), (0, 0)])
def test_reference_terrain_4k(fs, orc, gpu_ctx, hf, cf):
    d = _ref_maps()
    if not (d / "D1_4k.png").exists():
        pytest.skip("D1_4k.png not present")
    hm = (fs.png_read(d / "D1_4k.png") & 0xFF).astype(np.uint8)
    assert hm.shape == (4096, 4096)
    cm = fs.gen_colors(33, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params(height_filter=hf, color_filter=cf)
    op = orc.params_from(p)
    views = [(c, 2560, 1440) for c in fs.gen_cameras(34, hm, 2, above=(20, 200),
                                                      distance=(3000, 3000), screen_h=1440)]
    for cam, w, h in views:
        got = gpu_ctx.render(fmap, cam, w, h, params=p)
        want = orc.render(cam, op, hm, cm, w, h, threads=0)
        assert count_diff(got, want) == 0, (w, h, cam.as_tuple())
    # the same views batched in one plan
    plan = fs.Plan(gpu_ctx, [fmap], views, params=p)
    plan.run()
    for (cam, w, h), got in zip(views, plan.frames()):
        want = orc.render(cam, op, hm, cm, w, h, threads=0)
        assert count_diff(got, want) == 0
    plan.close()
    fmap.close()
