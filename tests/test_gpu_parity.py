"""GPU parity: every frame the CUDA path renders equals the CPU oracle's, bit
for bit (integer/byte output: no tolerance). Calls go through the C ABI."""
import numpy as np
import pytest

from conftest import count_diff

pytestmark = pytest.mark.gpu

FILTERS = [(h, c) for h in (0, 1) for c in (0, 1)]


def _params(fs, **kw):
    return fs.default_params(**kw)


@pytest.mark.parametrize("hf,cf", FILTERS)
def test_small_frames_all_filters(fs, orc, gpu_ctx, maps256, hf, cf):
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    cams = fs.gen_cameras(31, hm, 6, above=(20, 80), distance=(150, 500), screen_h=48)
    for cam in cams:
        p = _params(fs, height_filter=hf, color_filter=cf)
        got = gpu_ctx.render(fmap, cam, 64, 48, params=p)
        ref = orc.render(cam, orc.params_from(p), hm, cm, 64, 48)
        assert count_diff(got, ref) == 0


def test_config1_frame(fs, orc, gpu_ctx, maps1024):
    """320x240, 1024^2 map, D=800 (n=1265), camera 40 above the local maximum."""
    hm, cm = maps1024
    fmap = fs.Map(gpu_ctx, hm, cm)
    for cam in fs.gen_cameras(41, hm, 8, above=(40, 40), distance=(800, 800), screen_h=240):
        got = gpu_ctx.render(fmap, cam, 320, 240)
        ref = orc.render(cam, orc.make_params(), hm, cm, 320, 240, threads=0)
        assert count_diff(got, ref) == 0
