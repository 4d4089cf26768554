"""CPU oracle for the voxel-space render path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, and only as the checker (or the timed CPU stand-in). The product
(futspace_gb300/) never imports it.

PARITY UNPINNED: the reference ships no golden outputs and its Futhark sources
cannot be compiled here (no `futhark` compiler; lys/matte/linalg are not
vendored). Two independent restatements of the reference arithmetic are kept:

* fs_oracle.c (this package's C library): the reference pipeline column by
  column -- [n][w] samples, inclusive `occlude` scan, scatter, `fill_vline` scan,
  sky, transpose (fut/voxel_renderer.fut:214-251);
* literal.py: the same pipeline vectorised over whole arrays in numpy float32.

The tests require the two to agree bit for bit before either is trusted.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
LIB_PATH = _DIR / "_build" / "libfs_oracle.so"
NEAREST, BILINEAR = 0, 1
GAP_ZERO, GAP_SKY = 0, 1


class OCamera(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("height", C.c_float), ("angle", C.c_float),
                ("horizon", C.c_float), ("distance", C.c_float), ("fov", C.c_float),
                ("sky_color", C.c_uint32)]


class OParams(C.Structure):
    _fields_ = [("d", C.c_float), ("z0", C.c_float), ("scale", C.c_float),
                ("height_filter", C.c_int32), ("color_filter", C.c_int32),
                ("gap_rule", C.c_int32), ("floor_n", C.c_int32), ("effects", C.c_int32),
                ("shade", C.c_float), ("fog_start", C.c_float), ("fog_end", C.c_float),
                ("fog_color", C.c_uint32), ("smoothing", C.c_int32)]


_LIB = None


def build() -> Path:
    src = _DIR / "fs_oracle.c"
    LIB_PATH.parent.mkdir(exist_ok=True)
    if LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= max(
            src.stat().st_mtime, (_DIR / "fs_oracle.h").stat().st_mtime):
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(".so.tmp")
    subprocess.run(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off",
                    "-fopenmp", str(src), "-o", str(tmp), "-lm"], check=True)
    tmp.replace(LIB_PATH)
    return LIB_PATH


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(str(build()))
        P = C.POINTER
        f32, i32, u32, vp = C.c_float, C.c_int32, C.c_uint32, C.c_void_p
        for name, res, args in [
            ("fso_f2i", i32, [f32]), ("fso_f2u", u32, [f32]), ("fso_mod", i32, [i32, i32]),
            ("fso_mix", u32, [f32, u32, f32, u32]), ("fso_scale", u32, [u32, f32]),
            ("fso_num_depths", i32, [f32, f32, f32, i32]),
            ("fso_get_zs", i32, [f32, f32, f32, i32, vp, i32]),
            ("fso_height_bilinear", f32, [vp, i32, i32, f32, f32]),
            ("fso_height_nearest", f32, [vp, i32, i32, f32, f32]),
            ("fso_color_bilinear", u32, [vp, i32, i32, f32, f32]),
            ("fso_color_nearest", u32, [vp, i32, i32, f32, f32]),
            ("fso_render", i32, [P(OCamera), P(OParams), vp, vp, i32, i32, i32, i32, vp]),
            ("fso_render_mt", i32, [P(OCamera), P(OParams), vp, vp, i32, i32, i32, i32, vp, i32]),
            ("fso_max_threads", i32, []),
            ("fso_render_split", i32, [P(OCamera), P(OParams), vp, i32, i32, vp, i32, i32, i32,
                                       i32, vp, i32]),
            ("fso_shadowmap", i32, [vp, vp, i32, i32, vp, vp, i32]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def to_ocam(cam) -> OCamera:
    """Accepts any object with the camera fields (futspace_gb300.Camera, a dict)."""
    get = (lambda k: cam[k]) if isinstance(cam, dict) else (lambda k: getattr(cam, k))
    return OCamera(*(get(k) for k in ("x", "y", "height", "angle", "horizon", "distance", "fov",
                                      "sky_color")))


def make_params(d=0.001, z0=0.0, scale=0.0, height_filter=BILINEAR, color_filter=BILINEAR,
                gap_rule=GAP_ZERO, floor_n=1, effects=0, shade=0.0, fog_start=0.0, fog_end=0.0,
                fog_color=0, smoothing=0) -> OParams:
    return OParams(d, z0, scale, height_filter, color_filter, gap_rule, floor_n, effects, shade,
                   fog_start, fog_end, fog_color, smoothing)


def params_from(p) -> OParams:
    """From a futspace_gb300.Params."""
    return make_params(p.invz_param1, p.invz_param2, p.magic_number, p.height_filter,
                       p.color_filter, p.gap_rule, p.floor_n, p.effects, p.shade, p.fog_start,
                       p.fog_end, p.fog_color, getattr(p, "smoothing", 0))


def render(cam, params: OParams, heights: np.ndarray, colors: np.ndarray, width: int,
           height: int, threads: int = 1) -> np.ndarray:
    h = np.ascontiguousarray(heights, np.uint8)
    c = np.ascontiguousarray(colors, np.uint32)
    out = np.empty((height, width), np.uint32)
    oc = to_ocam(cam)
    if h.shape != c.shape:
        rc = lib().fso_render_split(C.byref(oc), C.byref(params), h.ctypes.data, h.shape[0],
                                    h.shape[1], c.ctypes.data, c.shape[0], c.shape[1], width,
                                    height, out.ctypes.data, threads)
    elif threads == 1:
        rc = lib().fso_render(C.byref(oc), C.byref(params), h.ctypes.data, c.ctypes.data,
                              h.shape[0], h.shape[1], width, height, out.ctypes.data)
    else:
        rc = lib().fso_render_mt(C.byref(oc), C.byref(params), h.ctypes.data, c.ctypes.data,
                                 h.shape[0], h.shape[1], width, height, out.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"oracle render failed ({rc})")
    return out


def get_zs(D: float, d: float = 0.001, z0: float = 0.0, floor_n: int = 1) -> np.ndarray:
    n = lib().fso_num_depths(D, d, z0, floor_n)
    if n < 1:
        return np.zeros(0, np.float32)
    out = np.empty(n, np.float32)
    lib().fso_get_zs(D, d, z0, floor_n, out.ctypes.data, n)
    return out


def shadowmap(heights: np.ndarray, colors: np.ndarray, sun, threads: int = 0) -> np.ndarray:
    h = np.ascontiguousarray(heights, np.uint8)
    c = np.ascontiguousarray(colors, np.uint32)
    s = np.asarray(sun, np.float32)
    out = np.empty((1024, 1024), np.uint32)
    rc = lib().fso_shadowmap(h.ctypes.data, c.ctypes.data, h.shape[0], h.shape[1],
                             s.ctypes.data, out.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError("oracle shadowmap failed")
    return out
