"""The allocation-free render entry point, fs_render_device_noalloc.

It exists for callers that cannot let a library call cudaMalloc -- hosts that
own all device memory through their own pool, or per-frame loops that cannot
take the device synchronisation an allocation may cause. Its only scratch is a
fixed array compiled into the library. Called through the C ABI; its frames must
equal fs_render_device's bit for bit (the tests' tolerance for u32 frames), on
two calls in a row, and it must not change the device's free memory.

Collected last (file name), so a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import count_diff

pytestmark = pytest.mark.gpu


def test_noalloc_matches_render_device(fs, gpu_ctx):
    torch = pytest.importorskip("torch")
    L = fs.lib()
    fn = L.fs_render_device_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(fs.Camera), C.POINTER(fs.Params), C.c_int32,
                   C.c_int32, C.c_void_p]
    hm = fs.gen_heights(5, 1024, 0.55)
    cm = fs.gen_colors(6, hm, 12)
    fmap = fs.Map(gpu_ctx, hm, cm)
    p = fs.default_params()
    cams = fs.gen_cameras(7, hm, 2, above=(20, 120), distance=(800, 3000), screen_h=480)
    ref = torch.empty((480, 640), dtype=torch.int32, device="cuda")
    got = torch.empty((480, 640), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for i, cam in enumerate(cams):  # two calls in a row, different cameras
        gpu_ctx.render_device(fmap, cam, 640, 480, ref, params=p)
        gpu_ctx.sync()
        got.fill_(0)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = fn(gpu_ctx.handle, fmap.handle, C.byref(cam), C.byref(p), 640, 480, got.data_ptr())
        assert rc == 0, gpu_ctx.error()
        gpu_ctx.sync()
        assert torch.cuda.mem_get_info()[0] == free_before  # nothing was allocated
        a = ref.cpu().numpy().view(np.uint32)
        b = got.cpu().numpy().view(np.uint32)
        assert count_diff(a, b) == 0, i
    # beyond the stated maximum: a clear error, no launch
    far = fs.Camera(*cams[0].as_tuple())
    far.distance = 5.0e6
    rc = fn(gpu_ctx.handle, fmap.handle, C.byref(far), C.byref(p), 640, 480, got.data_ptr())
    assert rc == 1 and "at most 65536" in gpu_ctx.error()
    fmap.close()
