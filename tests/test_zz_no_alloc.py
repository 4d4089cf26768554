"""The allocation-free render entry point, fs_render_device_noalloc.

It exists for callers that cannot let a library call cudaMalloc -- hosts that
own all device memory through their own pool, or per-frame loops that cannot
take the device synchronisation an allocation may cause. Its only scratch is a
fixed array compiled into the library. Called through the C ABI; its frames must
equal fs_render_device's and the CPU oracle's bit for bit (the tests' tolerance
for u32 frames: 0 differing pixels), on two calls in a row, and it must not
change the device's free memory. One frame uses a depth count just under the
array's 65536-entry limit, so the array's top entries and its zero padding are
read.

Collected last (file name), so a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import count_diff

pytestmark = pytest.mark.gpu

MAX_DEPTHS = 65536


def _entry(fs):
    fn = fs.lib().fs_render_device_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(fs.Camera), C.POINTER(fs.Params), C.c_int32,
                   C.c_int32, C.c_void_p]
    return fn


def _render_both(fs, orc, gpu_ctx, fn, fmap, hm, cm, cams, W, H):
    torch = pytest.importorskip("torch")
    p = fs.default_params()
    ref = torch.empty((H, W), dtype=torch.int32, device="cuda")
    got = torch.empty((H, W), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for i, cam in enumerate(cams):  # calls in a row, different cameras
        gpu_ctx.render_device(fmap, cam, W, H, ref, params=p)
        gpu_ctx.sync()
        got.fill_(0)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = fn(gpu_ctx.handle, fmap.handle, C.byref(cam), C.byref(p), W, H, got.data_ptr())
        assert rc == 0, gpu_ctx.error()
        gpu_ctx.sync()
        assert torch.cuda.mem_get_info()[0] == free_before  # nothing was allocated
        a = ref.cpu().numpy().view(np.uint32)
        b = got.cpu().numpy().view(np.uint32)
        assert count_diff(a, b) == 0, i
        want = orc.render(cam, orc.params_from(p), hm, cm, W, H, threads=0)
        assert count_diff(b, want) == 0, i
    return got


def test_noalloc_matches_render_device_and_oracle(fs, orc, gpu_ctx):
    fn = _entry(fs)
    hm = fs.gen_heights(5, 1024, 0.55)
    cm = fs.gen_colors(6, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    cams = fs.gen_cameras(7, hm, 2, above=(20, 120), distance=(800, 3000), screen_h=480)
    got = _render_both(fs, orc, gpu_ctx, fn, fmap, hm, cm, cams, 640, 480)
    # beyond the stated maximum: a clear error, no launch
    p = fs.default_params()
    far = fs.Camera(*cams[0].as_tuple())
    far.distance = 5.0e6
    rc = fn(gpu_ctx.handle, fmap.handle, C.byref(far), C.byref(p), 640, 480, got.data_ptr())
    assert rc == 1 and "at most 65536" in gpu_ctx.error()
    fmap.close()


def test_noalloc_near_depth_limit(fs, orc, gpu_ctx):
    """Two frames whose depth counts sit just under the fixed array's limit."""
    fn = _entry(fs)
    hm = fs.gen_heights(15, 1024, 0.55)
    cm = fs.gen_colors(16, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    # the largest draw distance whose schedule fits (n grows as sqrt(2000 D))
    D = 65535.0 ** 2 / 2000.0
    while fs.num_depths(D) > MAX_DEPTHS - 1:
        D *= 0.9999
    cams = fs.gen_cameras(17, hm, 2, above=(10, 60), distance=(D, D), screen_h=64)
    n = fs.num_depths(D)
    assert MAX_DEPTHS - 64 <= n <= MAX_DEPTHS - 1, n
    _render_both(fs, orc, gpu_ctx, fn, fmap, hm, cm, cams, 96, 64)
    fmap.close()
