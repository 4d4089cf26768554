"""Seeded synthetic inputs restated in numpy -- TEST INFRASTRUCTURE ONLY.

The same bytes as the product library's generators (diamond-square height
maps, palette colour maps, cameras, camera walks), computed without loading
that library, so the CPU reference arm of the benchmark and the oracle-side
checks need nothing from the product. tests/test_oracle_gen.py holds the two
to the committed digests in tests/golden/generators.txt and to each other.

The pseudo-random stream is splitmix64: output k of a stream seeded with s is
mix(s + (k + 1) * 0x9E3779B97F4A7C15), so the draws of a whole level of the
diamond-square recursion, or of a whole colour map, are computed at once from
their positions in the stream. Floating-point steps use float32 or float64
exactly where the generators' definition does (numpy rounds every operation to
its dtype, as C does with contraction off).

Definitions (the workloads' shapes): heights are a toroidal diamond-square map
with amplitude 1 halved by `roughness` per level, rescaled to 0..255 with
round-half-up; colours follow a 5-stop palette (deep water, sand, grass, rock,
snow) indexed by height, plus uniform integer noise in [-noise, noise] per
channel, alpha 0xFF; a camera stands uniform on the map, yaw uniform in
[0, 2 pi), height above the 16x16 local maximum uniform in [lo, hi], draw
distance uniform in [dlo, dhi], horizon screen_h / 2, fov 1.2, sky 0xFF9090E0.
"""
from __future__ import annotations

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
TWO_PI = 6.283185307179586
STOPS = np.array([[0, 24, 52, 120], [72, 196, 178, 128], [120, 62, 138, 52],
                  [190, 116, 104, 92], [255, 246, 246, 250]], np.int64)
SKY = 0xFF9090E0


class Stream:
    """A splitmix64 stream; take(k) returns its next k outputs as uint64."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.pos = 0

    def take(self, k: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            i = np.arange(self.pos + 1, self.pos + 1 + k, dtype=np.uint64)
            z = self.state + i * GAMMA
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            z = z ^ (z >> np.uint64(31))
        self.pos += k
        return z

    def u01(self, k: int) -> np.ndarray:
        """k uniforms in [0, 1) from the top 53 bits, as float64."""
        return (self.take(k) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def heights(seed: int, size: int, roughness: float = 0.55) -> np.ndarray:
    """[size][size] u8 diamond-square heights (size a power of two)."""
    if size < 2 or size & (size - 1):
        raise ValueError("size must be a power of two >= 2")
    N = size
    f = np.zeros((N, N), np.float32)
    s = Stream(seed ^ 0x5EED0F7E11A1)
    amp = np.float32(1.0)
    rough = np.float32(roughness)
    q = np.float32(0.25)
    step = N
    while step > 1:
        half = step // 2
        # diamond: the centre of every step x step square, rows then columns
        ys = np.arange(0, N, step)
        c00 = f[np.ix_(ys, ys)]
        c01 = f[np.ix_(ys, (ys + step) % N)]
        c10 = f[np.ix_((ys + step) % N, ys)]
        c11 = f[np.ix_((ys + step) % N, (ys + step) % N)]
        avg = (((c00 + c01) + c10) + c11) * q
        r = (s.u01(len(ys) * len(ys)) * 2.0 - 1.0).astype(np.float32).reshape(len(ys), len(ys))
        f[np.ix_(ys + half, ys + half)] = avg + r * amp
        # square: edge midpoints, rows y = 0, half, 2 half, ... in order; in
        # row y the points start at x = half when y / half is even, else 0
        rows = np.arange(0, N, half)
        npr = N // step  # points per row
        r = (s.u01(len(rows) * npr) * 2.0 - 1.0).astype(np.float32).reshape(len(rows), npr)
        for parity in (0, 1):
            ry = rows[(rows // half) % 2 == parity]
            xs = np.arange(half if parity == 0 else 0, N, step)
            a = f[np.ix_((ry - half) % N, xs)]
            b = f[np.ix_((ry + half) % N, xs)]
            c = f[np.ix_(ry, (xs - half) % N)]
            d = f[np.ix_(ry, (xs + half) % N)]
            avg = (((a + b) + c) + d) * q
            f[np.ix_(ry, xs)] = avg + r[(ry // half)] * amp
        amp = np.float32(amp * rough)
        step = half
    mn, mx = float(f.min()), float(f.max())
    span = mx - mn
    if span > 0.0:
        v = (f.astype(np.float64) - mn) / span * 255.0
        b = (v + 0.5).astype(np.int64)
    else:
        b = np.zeros((N, N), np.int64)
    return np.clip(b, 0, 255).astype(np.uint8)


def colors(seed: int, hmap: np.ndarray, noise: int = 12) -> np.ndarray:
    """ARGB u32 colours from the palette of the heights, plus channel noise."""
    h = np.ascontiguousarray(hmap, np.uint8)
    flat = h.reshape(-1).astype(np.int64)
    seg = np.zeros(flat.shape, np.int64)
    for k in range(3):
        seg += (flat > STOPS[k + 1, 0]) & (seg == k)
    h0, h1 = STOPS[seg, 0], STOPS[seg + 1, 0]
    span, t = h1 - h0, flat - h0
    draws = Stream(seed ^ 0xC01065EED).take(3 * flat.size).reshape(-1, 3)
    mod = np.uint64(2 * noise + 1)
    out = np.full(flat.shape, 0xFF000000, np.uint64)
    for ch, shift in ((0, 16), (1, 8), (2, 0)):
        v = (STOPS[seg, ch + 1] * (span - t) + STOPS[seg + 1, ch + 1] * t + span // 2) // span
        v = v + (draws[:, ch] % mod).astype(np.int64) - noise
        out |= np.clip(v, 0, 255).astype(np.uint64) << np.uint64(shift)
    return out.astype(np.uint32).reshape(h.shape)


def local_max(hmap: np.ndarray, x: float, y: float) -> int:
    """Maximum height over the 16x16 texels around (floor x, floor y), wrapping."""
    rows, cols = hmap.shape
    ix, iy = int(np.floor(np.float32(x))), int(np.floor(np.float32(y)))
    ys = (iy + np.arange(-8, 8)) % rows
    xs = (ix + np.arange(-8, 8)) % cols
    return int(hmap[np.ix_(ys, xs)].max())


def _camera(x, y, height, angle, horizon, distance) -> dict:
    f = lambda v: float(np.float32(v))  # noqa: E731  (a camera holds f32 fields)
    return {"x": f(x), "y": f(y), "height": f(height), "angle": f(angle), "horizon": f(horizon),
            "distance": f(distance), "fov": f(1.2), "sky_color": SKY}


def cameras(seed: int, hmap: np.ndarray, count: int, above=(40.0, 40.0),
            distance=(800.0, 800.0), screen_h: int = 240) -> list[dict]:
    """`count` cameras (dicts with the camera record's fields)."""
    rows, cols = hmap.shape
    f32 = lambda v: float(np.float32(v))  # noqa: E731
    lo, hi = f32(above[0]), f32(above[1])
    dlo, dhi = f32(distance[0]), f32(distance[1])
    u = Stream(seed ^ 0xCA3E7A5).u01(5 * count).reshape(count, 5) if count else np.zeros((0, 5))
    out = []
    for i in range(count):
        x, y = f32(u[i, 0] * cols), f32(u[i, 1] * rows)
        ang = u[i, 2] * TWO_PI
        ab = lo + u[i, 3] * (hi - lo)
        h = float(local_max(hmap, x, y)) + ab
        d = dlo + u[i, 4] * (dhi - dlo)
        out.append(_camera(x, y, h, ang, screen_h // 2, d))
    return out


def _sincos(a: float):
    """sin and cos by reduction to [-pi, pi] and 13 Taylor terms each (the walk's
    definition; the renderer never uses it)."""
    two_pi, pi = 6.283185307179586476925, 3.141592653589793238463
    k = float(int(a / two_pi))
    r = a - k * two_pi
    while r > pi:
        r -= two_pi
    while r < -pi:
        r += two_pi
    r2 = r * r
    term = s = r
    for i in range(1, 14):
        term = -term * r2 / float((2 * i) * (2 * i + 1))
        s = s + term
    term = c = 1.0
    for i in range(1, 14):
        term = -term * r2 / float((2 * i - 1) * (2 * i))
        c = c + term
    return s, c


def walk(seed: int, hmap: np.ndarray, count: int, step: float = 2.0, yaw: float = 0.02,
         above=(30.0, 120.0), distance: float = 3000.0, screen_h: int = 1080) -> list[dict]:
    """A camera random walk: each frame turns by U(-yaw, yaw), moves `step`
    forward along (-sin, -cos) and keeps its height within [lo, hi] above the
    local maximum (the height offset moves by U(-5, 5) per frame)."""
    rows, cols = hmap.shape
    f32 = lambda v: float(np.float32(v))  # noqa: E731
    step, yaw = f32(step), f32(yaw)
    lo, hi = f32(above[0]), f32(above[1])
    s = Stream(seed ^ 0x3A1C3A1C)
    x, y = s.u01(1)[0] * cols, s.u01(1)[0] * rows
    ang = s.u01(1)[0] * TWO_PI
    ab = (lo + hi) * 0.5
    out = []
    for i in range(count):
        if i > 0:
            ang = ang + (s.u01(1)[0] * 2.0 - 1.0) * yaw
            sn, cs = _sincos(ang)
            x = x - step * sn
            y = y - step * cs
            ab = min(max(ab + (s.u01(1)[0] * 2.0 - 1.0) * 5.0, lo), hi)
        cx, cy = f32(x), f32(y)
        out.append(_camera(cx, cy, float(local_max(hmap, cx, cy)) + ab, ang, screen_h // 2,
                           distance))
    return out


def camera_bytes(cams: list[dict]) -> bytes:
    """The cameras as packed camera records (7 f32 + u32 each)."""
    rec = np.zeros(len(cams), dtype=[("x", "<f4"), ("y", "<f4"), ("height", "<f4"),
                                     ("angle", "<f4"), ("horizon", "<f4"), ("distance", "<f4"),
                                     ("fov", "<f4"), ("sky_color", "<u4")])
    for i, c in enumerate(cams):
        for k in rec.dtype.names:
            rec[i][k] = c[k]
    return rec.tobytes()
