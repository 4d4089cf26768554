"""The Futhark-compatible entry points (include/libfutspace.h), called through
the C ABI the way c/interactive.c and lys call them: init, resize,
update_map, key, step, text_content, render, values. Frames are checked bit
for bit against the oracle (shadow-map precompute + render)."""
import ctypes as C

import numpy as np
import pytest

from conftest import count_diff

pytestmark = pytest.mark.gpu

f32 = np.float32
_libm = C.CDLL("libm.so.6")
for _n in ("sinf", "cosf"):
    getattr(_libm, _n).restype = C.c_float
    getattr(_libm, _n).argtypes = [C.c_float]


def _api(fs):
    L = C.CDLL(str(fs.library_path()))
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    P = C.POINTER
    sig = {
        "futhark_context_config_new": (vp, []),
        "futhark_context_config_set_device": (None, [vp, C.c_char_p]),
        "futhark_context_config_free": (None, [vp]),
        "futhark_context_new": (vp, [vp]),
        "futhark_context_free": (None, [vp]),
        "futhark_context_sync": (C.c_int, [vp]),
        "futhark_context_get_error": (vp, [vp]),
        "futhark_new_u32_2d": (vp, [vp, vp, i64, i64]),
        "futhark_new_i32_2d": (vp, [vp, vp, i64, i64]),
        "futhark_free_u32_2d": (C.c_int, [vp, vp]),
        "futhark_free_i32_2d": (C.c_int, [vp, vp]),
        "futhark_values_u32_2d": (C.c_int, [vp, vp, vp]),
        "futhark_shape_u32_2d": (P(i64), [vp, vp]),
        "futhark_free_opaque_state": (C.c_int, [vp, vp]),
        "futhark_entry_init": (C.c_int, [vp, P(vp), C.c_uint32]),
        "futhark_entry_resize": (C.c_int, [vp, P(vp), i32, i32, vp]),
        "futhark_entry_key": (C.c_int, [vp, P(vp), i32, i32, vp]),
        "futhark_entry_mouse": (C.c_int, [vp, P(vp), i32, i32, i32, vp]),
        "futhark_entry_wheel": (C.c_int, [vp, P(vp), i32, i32, vp]),
        "futhark_entry_step": (C.c_int, [vp, P(vp), C.c_float, vp]),
        "futhark_entry_render": (C.c_int, [vp, P(vp), vp]),
        "futhark_entry_text_content": (C.c_int, [vp] + [P(C.c_float)] * 9 + [vp]),
        "futhark_entry_update_map": (C.c_int, [vp, P(vp), vp, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


class App:
    """A minimal stand-in for the lys loop: every entry returns a new state and
    the old one is freed, as the generated API requires."""

    def __init__(self, fs):
        self.L = _api(fs)
        cfg = self.L.futhark_context_config_new()
        self.L.futhark_context_config_set_device(cfg, b"0")
        self.ctx = self.L.futhark_context_new(cfg)
        self.cfg = cfg
        assert self.ctx
        self.state = C.c_void_p()
        self.ok(self.L.futhark_entry_init(self.ctx, C.byref(self.state), 7))

    def ok(self, rc):
        if rc != 0:
            p = self.L.futhark_context_get_error(self.ctx)
            msg = C.string_at(p).decode() if p else ""
            raise AssertionError(f"rc={rc}: {msg}")

    def apply(self, fn, *args):
        new = C.c_void_p()
        self.ok(fn(self.ctx, C.byref(new), *args, self.state))
        self.L.futhark_free_opaque_state(self.ctx, self.state)
        self.state = new

    def text(self):
        vals = [C.c_float() for _ in range(9)]
        self.ok(self.L.futhark_entry_text_content(self.ctx, *[C.byref(v) for v in vals],
                                                  self.state))
        return [v.value for v in vals]

    def render(self):
        arr = C.c_void_p()
        self.ok(self.L.futhark_entry_render(self.ctx, C.byref(arr), self.state))
        shape = self.L.futhark_shape_u32_2d(self.ctx, arr)
        h, w = shape[0], shape[1]
        out = np.empty((h, w), np.uint32)
        self.ok(self.L.futhark_values_u32_2d(self.ctx, arr, out.ctypes.data))
        self.L.futhark_free_u32_2d(self.ctx, arr)
        return out

    def close(self):
        self.L.futhark_free_opaque_state(self.ctx, self.state)
        self.L.futhark_context_free(self.ctx)
        self.L.futhark_context_config_free(self.cfg)


def sun_vector(sun_height, sun_ang):
    """vec3_rotate #y sun_ang (vec3_rotate #z sun_height [0,1,0]) in f32."""
    ch, sh = f32(_libm.cosf(f32(sun_height))), f32(_libm.sinf(f32(sun_height)))
    v1 = [f32(f32(f32(0) + ch * f32(0)) + f32(-sh) * f32(1)) + f32(0) * f32(0),
          f32(f32(f32(0) + sh * f32(0)) + ch * f32(1)) + f32(0) * f32(0),
          f32(f32(f32(0) + f32(0) * f32(0)) + f32(0) * f32(1)) + f32(1) * f32(0)]
    ca, sa = f32(_libm.cosf(f32(sun_ang))), f32(_libm.sinf(f32(sun_ang)))
    ry = [[ca, f32(0), sa], [f32(0), f32(1), f32(0)], [f32(-sa), f32(0), ca]]
    return np.array([f32(f32(f32(f32(0) + ry[i][0] * v1[0]) + ry[i][1] * v1[1]) + ry[i][2] * v1[2])
                     for i in range(3)], np.float32)


def test_interactive_session(fs, orc):
    try:
        app = App(fs)
    except AssertionError as e:
        pytest.skip(f"no CUDA device: {e}")
    try:
        # map load, as c/interactive.c:50-56 does
        hm = fs.gen_heights(41, 256, 0.55)
        cm = fs.gen_colors(42, hm, 12)
        hi = hm.astype(np.int32) | np.int32(0x3C00)  # update_map keeps the low byte
        ca = app.L.futhark_new_u32_2d(app.ctx, cm.ctypes.data, 256, 256)
        ha = app.L.futhark_new_i32_2d(app.ctx, hi.ctypes.data, 256, 256)
        app.apply(app.L.futhark_entry_update_map, ca, ha)
        app.L.futhark_free_u32_2d(app.ctx, ca)
        app.L.futhark_free_i32_2d(app.ctx, ha)
        app.apply(app.L.futhark_entry_resize, 120, 160)  # h, w

        def expected_frame(sun_h, sun_a, sky):
            shadow = orc.shadowmap(hm, cm, sun_vector(sun_h, sun_a), threads=0)
            x, y, ang, height, hor, dist, _, _, fov = app.text()
            cam = dict(x=x, y=y, height=height, angle=ang, horizon=hor, distance=dist, fov=fov,
                       sky_color=sky)
            return orc.render(cam, orc.make_params(), hm, shadow, 160, 120, threads=0)

        # fresh state: sky colour 0 until the first step
        assert count_diff(app.render(), expected_frame(0.1, 0.1, 0)) == 0

        # hold W (forward) for three steps, then release
        x0, y0 = app.text()[:2]
        app.apply(app.L.futhark_entry_key, 0, ord("w"))
        for _ in range(3):
            app.apply(app.L.futhark_entry_step, f32(0.016))
        app.apply(app.L.futhark_entry_key, 1, ord("w"))
        app.apply(app.L.futhark_entry_mouse, 1, 10, 10)
        app.apply(app.L.futhark_entry_wheel, 0, 1)
        x, y, ang = app.text()[:3]
        s, c = f32(_libm.sinf(f32(2.2))), f32(_libm.cosf(f32(2.2)))
        ex, ey = f32(x0), f32(y0)
        for _ in range(3):
            ex, ey = f32(ex - f32(3) * s), f32(ey - f32(3) * c)
        assert (x, y, ang) == (ex, ey, f32(2.2))
        sky = orc.lib().fso_scale(0xFF9090E0, 0.1)
        assert count_diff(app.render(), expected_frame(0.1, 0.1, sky)) == 0

        # U raises the sun; the shadow map is recomputed from the pre-step sun
        app.apply(app.L.futhark_entry_key, 0, ord("u"))
        app.apply(app.L.futhark_entry_step, f32(0.016))
        app.apply(app.L.futhark_entry_key, 1, ord("u"))
        sun_h = app.text()[6]
        assert sun_h == f32(f32(0.1) + f32(0.005))
        assert count_diff(app.render(), expected_frame(0.1, 0.1, sky)) == 0
        # one more step: sky follows the new sun height; shadow map unchanged
        app.apply(app.L.futhark_entry_step, f32(0.016))
        sky2 = orc.lib().fso_scale(0xFF9090E0, float(sun_h))
        assert count_diff(app.render(), expected_frame(0.1, 0.1, sky2)) == 0

        # raise the camera (R) and pitch (Q), then turn (A)
        for k in (ord("r"), ord("q"), ord("a")):
            app.apply(app.L.futhark_entry_key, 0, k)
        app.apply(app.L.futhark_entry_step, f32(0.016))
        for k in (ord("r"), ord("q"), ord("a")):
            app.apply(app.L.futhark_entry_key, 1, k)
        t = app.text()
        assert t[2] == f32(f32(2.2) + f32(0.10)) and t[4] == 220.0
        assert count_diff(app.render(), expected_frame(0.1, 0.1, sky2)) == 0

        # key 2 toggles the `#on` smoothing branch
        app.apply(app.L.futhark_entry_key, 0, ord("2"))
        app.apply(app.L.futhark_entry_step, f32(0.016))
        app.apply(app.L.futhark_entry_key, 1, ord("2"))
        shadow = orc.shadowmap(hm, cm, sun_vector(0.1, 0.1), threads=0)
        x, y, ang, height, hor, dist, _, _, fov = app.text()
        cam = dict(x=x, y=y, height=height, angle=ang, horizon=hor, distance=dist, fov=fov,
                   sky_color=sky2)
        want = orc.render(cam, orc.make_params(smoothing=1), hm, shadow, 160, 120, threads=0)
        assert count_diff(app.render(), want) == 0
        # math mode (key 1) is not provided: render reports an error instead of pixels
        app.apply(app.L.futhark_entry_key, 0, ord("1"))
        app.apply(app.L.futhark_entry_step, f32(0.016))
        app.apply(app.L.futhark_entry_key, 1, ord("1"))
        with pytest.raises(AssertionError, match="math mode"):
            app.render()
    finally:
        app.close()
