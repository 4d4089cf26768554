"""Second, independent restatement of the reference render -- TEST INFRASTRUCTURE ONLY.

PARITY UNPINNED (no reference outputs exist). This one follows the Futhark
source as whole-array operations in numpy float32, one array expression per
source line, so it shares no code with fs_oracle.c. Small cases only.

Only sin/cos/pow come from the C library (via ctypes): those are the libm calls
a `futhark c` build makes for f32.sin, f32.cos and `**`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

f32 = np.float32
_libm = C.CDLL("libm.so.6")
for _n in ("sinf", "cosf"):
    getattr(_libm, _n).restype = C.c_float
    getattr(_libm, _n).argtypes = [C.c_float]
_libm.powf.restype = C.c_float
_libm.powf.argtypes = [C.c_float, C.c_float]

I32_MAX, I32_MIN = 2147483647, -2147483648


def f2i(a) -> np.ndarray:
    """i32.f32 with the saturating GPU rule: NaN -> 0, clamp, truncate."""
    a = np.asarray(a, np.float32).astype(np.float64)
    t = np.trunc(np.nan_to_num(a, nan=0.0, posinf=2.0**31, neginf=-(2.0**31)))
    return np.clip(t, I32_MIN, I32_MAX).astype(np.int64)


def f2u(a) -> np.ndarray:
    a = np.asarray(a, np.float32).astype(np.float64)
    t = np.trunc(np.nan_to_num(a, nan=0.0, posinf=2.0**32, neginf=0.0))
    return np.clip(t, 0, 2**32 - 1).astype(np.uint64)


def get_zs(c: float, d: float, z0: float, floor_n: int = 1) -> np.ndarray:
    """fut/voxel_renderer.fut:28-34"""
    c, d, z0 = f32(c), f32(d), f32(z0)
    sq = np.sqrt(f32(_libm.powf(f32(d - f32(2) * z0), 2.0)) + f32(8) * d * c, dtype=np.float32)
    num = f32(f32(sq - f32(2) * z0) + d)
    div = f32(f32(2) * d)
    q = f32(num / div)
    n = int(f2i(np.floor(q) if floor_n else q))
    if n < 1:
        return np.zeros(0, np.float32)
    i = np.arange(1, n + 1, dtype=np.float32)
    return (i / f32(2)) * (f32(2) * z0 + (i - f32(1)) * d)


def _to_rgba(c: np.ndarray):
    c = c.astype(np.uint32)
    return [((c >> np.uint32(s)) & np.uint32(0xFF)).astype(np.float32) / f32(255)
            for s in (16, 8, 0, 24)]


def _from_rgba(r, g, b, a):
    def byte(x):
        x = np.where(x < f32(0), f32(0), np.where(x > f32(1), f32(1), x)).astype(np.float32)
        return f2u(x * f32(255)).astype(np.uint32)
    return (byte(a) << np.uint32(24)) | (byte(r) << np.uint32(16)) | (byte(g) << np.uint32(8)) | byte(b)


def mix(w1, c1, w2, c2):
    """matte 0.1.2 colourspace.mix, restated (weights normalised by w1 + w2)."""
    with np.errstate(invalid="ignore", divide="ignore"):
        w1 = np.asarray(w1, np.float32)
        w2 = np.asarray(w2, np.float32)
        w1n = w1 / (w1 + w2)
        w2n = w2 / (w1 + w2)
        ch1, ch2 = _to_rgba(np.asarray(c1)), _to_rgba(np.asarray(c2))
        ch = [x1 * w1n + x2 * w2n for x1, x2 in zip(ch1, ch2)]
        return _from_rgba(*ch)


def _gather(m, iy, ix):
    return m[np.mod(iy, m.shape[0]), np.mod(ix, m.shape[1])]


def scale_colour(c, s):
    """matte colourspace.scale (RGB times s, alpha kept)."""
    r, g, b, a = _to_rgba(np.asarray(c))
    s = np.asarray(s, np.float32)
    return _from_rgba(r * s, g * s, b * s, a)


def _smooth(col, row, n, W, H, sky):
    """The `#on` branch, fut/voxel_renderer.fut:175-213, columns vectorised."""
    acc_c = np.zeros(W, np.uint32)
    acc_r = np.full(W, H, np.int64)
    acc_i = np.zeros(W, np.int64)
    sc = np.empty((n, W), np.uint32)
    sr = np.empty((n, W), np.int64)
    si = np.empty((n, W), np.int64)
    for k in range(n):  # scan occlude2 with neutral (0, h, 0)
        take = ~(acc_r <= row[k])
        acc_c = np.where(take, col[k], acc_c)
        acc_r = np.where(take, row[k], acc_r)
        acc_i = np.where(take, k, acc_i)
        sc[k], sr[k], si[k] = acc_c, acc_r, acc_i
    # rotate (-1): element k pairs with element k-1 (element 0 with element n-1)
    pc, pr, pi = np.roll(sc, 1, axis=0), np.roll(sr, 1, axis=0), np.roll(si, 1, axis=0)
    fields = [np.zeros((H, W), np.uint32), np.zeros((H, W), np.uint32),
              np.zeros((H, W), np.int64), np.zeros((H, W), np.int64),
              np.full((H, W), 1000, np.int64), np.full((H, W), 1000, np.int64)]
    cols = np.arange(W)
    for k in range(n):  # scatter, later indices overwrite earlier ones
        ok = sr[k] < H
        rr, cc = sr[k][ok], cols[ok]
        for f, v in zip(fields, (sc[k], pc[k], sr[k], pr[k], si[k], pi[k])):
            f[rr, cc] = v[ok]
    carry = [np.zeros(W, np.uint32), np.zeros(W, np.uint32), np.zeros(W, np.int64),
             np.zeros(W, np.int64), np.full(W, 1000, np.int64), np.full(W, 1000, np.int64)]
    out = np.empty((H, W), np.uint32)
    with np.errstate(invalid="ignore", divide="ignore"):
        for y in range(H):
            t = [f[y] for f in fields]
            empty = ((t[0] == 0) & (t[1] == 0) & (t[2] == 0) & (t[3] == 0) & (t[4] == 1000)
                     & (t[5] == 1000))
            carry = [np.where(empty, c, v) for c, v in zip(carry, t)]
            c0, c1, r2, r3, i4, i5 = carry
            rng = np.maximum(f32(1), (r3 - r2).astype(np.float32))
            d1 = np.abs(f32(y) - r3.astype(np.float32)) / rng
            d2 = np.abs(r2.astype(np.float32) - f32(y)) / rng
            c = np.where(i4 - i5 == 1, mix(d2, c1, d1, c0), c0).astype(np.uint32)
            out[y] = np.where(c == 0, sky, c)
    return out


def render(cam, hm, cm, W, H, d=0.001, z0=0.0, scale=0.0, height_filter=1, color_filter=1,
           gap_rule=0, floor_n=1, effects=0, shade=0.0, fog_start=0.0, fog_end=0.0,
           fog_color=0, smoothing=0) -> np.ndarray:
    """fut/voxel_renderer.fut:101-251 (`#off`) with the samplers of
    fut/render_functions.fut:63-105."""
    get = (lambda k: cam[k]) if isinstance(cam, dict) else (lambda k: getattr(cam, k))
    cx_, cy_, ch_, ang = f32(get("x")), f32(get("y")), f32(get("height")), get("angle")
    hor, D, fov, sky = f32(get("horizon")), f32(get("distance")), f32(get("fov")), get("sky_color")
    zs = get_zs(D, d, z0, floor_n)
    if zs.size == 0:
        raise ValueError("empty depth range")
    s, c = f32(_libm.sinf(f32(ang))), f32(_libm.cosf(f32(ang)))
    # get_h_line (:43-60), one row per z
    lx = (f32(-c) - s * fov) * zs
    ly = (s - c * fov) * zs
    rx = (c - s * fov) * zs
    ry = (f32(-s) - c * fov) * zs
    dx = (rx - lx) / f32(W)
    dy = (ry - ly) / f32(W)
    sx = lx + cx_
    sy = ly + cy_
    with np.errstate(divide="ignore"):
        inv_z = (f32(1) / zs) * (f32(scale) if scale > 0 else f32(W // 2))
    # get_segment (:63-66), [n][w]
    iw = np.arange(W, dtype=np.float32)[None, :]
    x = sx[:, None] + iw * dx[:, None]
    y = sy[:, None] + iw * dy[:, None]
    hm = np.asarray(hm, np.uint8)
    cm = np.asarray(cm, np.uint32)
    with np.errstate(invalid="ignore"):
        if height_filter:
            fx, cxx, fy, cyy = np.floor(x), np.ceil(x), np.floor(y), np.ceil(y)
            h = lambda yy, xx: _gather(hm, f2i(yy), f2i(xx)).astype(np.float32)
            x1 = (cxx - x) * h(fy, fx) + (x - fx) * h(fy, cxx)
            x2 = (cxx - x) * h(cyy, fx) + (x - fx) * h(cyy, cxx)
            mh = (cyy - y) * x1 + (y - fy) * x2
        else:
            mh = _gather(hm, f2i(y), f2i(x)).astype(np.float32)
        if color_filter:
            fx, cxx, fy, cyy = np.floor(x), np.ceil(x), np.floor(y), np.ceil(y)
            cc = lambda yy, xx: _gather(cm, f2i(yy), f2i(xx))
            c1 = mix(cxx - x, cc(fy, fx), x - fx, cc(fy, cxx))
            c2 = mix(cxx - x, cc(cyy, fx), x - fx, cc(cyy, cxx))
            col = mix(cyy - y, c1, y - fy, c2)
        else:
            col = _gather(cm, f2i(y), f2i(x)).astype(np.uint32)
        rel = (ch_ - mh) * inv_z[:, None] + hor
        zz = np.broadcast_to(zs[:, None], col.shape).astype(np.float32)
        if effects & 1:
            col = scale_colour(col, f32(1) - f32(shade) * (zz / D))
        if effects & 2:
            fo = (zz - f32(fog_start)) / (f32(fog_end) - f32(fog_start))
            fo = np.where(fo < f32(0), f32(0), np.where(fo > f32(1), f32(1), fo)).astype(np.float32)
            col = mix(f32(1) - fo, col, fo, np.uint32(fog_color))
    row = np.maximum(0, f2i(rel))
    if smoothing:
        return _smooth(col, row, zs.size, W, H, np.uint32(sky))
    # per column: scan occlude with neutral (0, h) (:231), scatter (:244),
    # scan fill_vline (:246), sky (:248); columns vectorised
    n = zs.size
    acc_c = np.zeros(W, np.uint32)
    acc_r = np.full(W, H, np.int64)
    sc = np.empty((n, W), np.uint32)
    sr = np.empty((n, W), np.int64)
    for k in range(n):
        take = ~(acc_r <= row[k])
        acc_c = np.where(take, col[k], acc_c)
        acc_r = np.where(take, row[k], acc_r)
        sc[k], sr[k] = acc_c, acc_r
    gap = np.uint32(sky if gap_rule else 0)
    vline = np.full((H, W), gap, np.uint32)
    cols = np.arange(W)
    for k in range(n):
        ok = sr[k] < H
        vline[sr[k][ok], cols[ok]] = sc[k][ok]
    out = np.empty((H, W), np.uint32)
    carry = np.full(W, gap, np.uint32)
    for yy in range(H):
        carry = np.where(vline[yy] != gap, vline[yy], carry)
        out[yy] = np.where(carry == gap, np.uint32(sky), carry)
    return out
