"""futspace_gb300 -- Voxel Space terrain renderer for one NVIDIA GB300 (sm_103a).

Python mirror of the C ABI in include/futspace_gb300.h, over ctypes. Every
render goes through the CUDA kernels in libfutspace_gb300.so; there is no CPU
fallback, and importing the renderer without the built library raises.

The renderer is the reference's per-frame ``render`` entry
(fut/interactive_entrypoints.fut:19-20 -> fut/interactive.fut:173-183 ->
fut/voxel_renderer.fut:101-251) with the samplers of
fut/render_functions.fut:63-105.
"""
from __future__ import annotations

import atexit
import ctypes as C
import sys
import weakref
from pathlib import Path
from typing import Iterable, Sequence

import numpy as np

__all__ = [
    "FsError", "Camera", "Params", "View", "Context", "Map", "Plan", "lib", "library_path",
    "default_params", "num_depths", "gen_heights", "gen_colors", "gen_cameras", "gen_walk",
    "local_max", "NEAREST", "BILINEAR", "GAP_ZERO", "GAP_SKY",
]

NEAREST, BILINEAR = 0, 1
GAP_ZERO, GAP_SKY = 0, 1
FX_SHADE, FX_FOG = 1, 2
_ERRORS = {1: "FS_ERR_ARG", 2: "FS_ERR_CUDA", 3: "FS_ERR_RANGE", 4: "FS_ERR_NOMEM",
           5: "FS_ERR_BUDGET", 6: "FS_ERR_STATE", 7: "FS_ERR_IO"}


class FsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRORS.get(code, code)}: {msg}")
        self.code = code


class Camera(C.Structure):
    """camera record, fut/voxel_renderer.fut:5-12"""
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("height", C.c_float), ("angle", C.c_float),
                ("horizon", C.c_float), ("distance", C.c_float), ("fov", C.c_float),
                ("sky_color", C.c_uint32)]

    def as_tuple(self):
        return tuple(getattr(self, f) for f, _ in self._fields_)


class Params(C.Structure):
    _fields_ = [("invz_param1", C.c_float), ("invz_param2", C.c_float),
                ("magic_number", C.c_float), ("height_filter", C.c_int32),
                ("color_filter", C.c_int32), ("gap_rule", C.c_int32), ("floor_n", C.c_int32),
                ("effects", C.c_int32), ("shade", C.c_float), ("fog_start", C.c_float),
                ("fog_end", C.c_float), ("fog_color", C.c_uint32), ("smoothing", C.c_int32)]


class Request(C.Structure):
    """fs_request: one render request of a serving session."""
    _fields_ = [("session", C.c_int32), ("map", C.c_int32), ("width", C.c_int32),
                ("height", C.c_int32), ("cam", Camera), ("host_out", C.c_void_p),
                ("arrival_ns", C.c_int64), ("start_ns", C.c_int64), ("done_ns", C.c_int64),
                ("status", C.c_int32), ("batch", C.c_int32)]


class ServerConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_int64), ("nsessions", C.c_int32), ("max_batch", C.c_int32),
                ("slots", C.c_int32), ("max_depths", C.c_int32), ("tune", C.c_int32 * 5)]


class ServeStats(C.Structure):
    _fields_ = [("wall_s", C.c_double), ("gpix_s", C.c_double), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double),
                ("requests", C.c_int64), ("pixels", C.c_int64), ("batches", C.c_int64),
                ("mean_batch", C.c_double), ("peak_arena_bytes", C.c_int64),
                ("max_inflight", C.c_int32), ("errors", C.c_int32),
                ("max_call_ms", C.c_double), ("max_call_site", C.c_int32),
                ("reserved", C.c_int32), ("max_sleep_ms", C.c_double),
                ("max_host_ms", C.c_double), ("max_batch_gpu_ms", C.c_double),
                ("max_batch_gpu_at_ns", C.c_int64), ("max_host_at_ns", C.c_int64),
                ("involuntary_switches", C.c_int64), ("voluntary_switches", C.c_int64)]

    SITES = {0: None, 1: "event query", 2: "copy in", 3: "counter reset", 4: "prologue launch",
             5: "render launch", 6: "frame copy out", 7: "event record"}

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}
        d["max_call_site"] = self.SITES.get(d["max_call_site"], d["max_call_site"])
        return d


class View(C.Structure):
    _fields_ = [("cam", Camera), ("width", C.c_int32), ("height", C.c_int32),
                ("map", C.c_int32), ("reserved", C.c_int32)]


def library_path() -> Path:
    return Path(__file__).resolve().parent / "_lib" / "libfutspace_gb300.so"


_LIB = None
# Live native objects, released in dependency order (servers, plans, pinned
# buffers, maps) at interpreter exit, while the CUDA runtime is still up;
# __del__ does nothing during finalisation. Contexts are only synchronised:
# their streams may be wrapped by other libraries' stream objects (a torch
# ExternalStream) whose pending uses are released after this handler, and
# destroying the stream first aborts those releases. Process teardown frees
# the contexts.
_LIVE: "weakref.WeakSet" = weakref.WeakSet()


def _release_all():
    objs = list(_LIVE)
    for o in objs:
        if isinstance(o, Context):
            try:
                o.sync()
            except Exception:
                pass
    for kind in (Server, Plan, PinnedBuffer, Map):
        for o in objs:
            if isinstance(o, kind):
                try:
                    o.close()
                except Exception:
                    pass


atexit.register(_release_all)


def _sig(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args


def lib():
    """The loaded native library; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        raise FsError(6, f"native library missing: {path} (run __graft_entry__.build())")
    L = C.CDLL(str(path))
    vp, i32, i64, u64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_float
    P = C.POINTER
    _sig(L, "fs_params_default", Params, [])
    _sig(L, "fs_ctx_new", C.c_int, [P(vp), i32])
    _sig(L, "fs_ctx_free", None, [vp])
    _sig(L, "fs_ctx_get_error", vp, [vp])
    _sig(L, "fs_ctx_sync", C.c_int, [vp])
    _sig(L, "fs_ctx_set_stream", C.c_int, [vp, vp])
    _sig(L, "fs_ctx_get_stream", vp, [vp])
    _sig(L, "fs_ctx_kernel_launches", i64, [vp])
    _sig(L, "fs_ctx_stats", C.c_int, [vp, i32, P(u64)])
    _sig(L, "fs_ctx_kernel_ms", C.c_int, [vp, P(C.c_float)])
    _sig(L, "fs_measure_l2_read_gbs", C.c_int, [vp, i64, i32, P(C.c_float)])
    _sig(L, "fs_ctx_force_tune", C.c_int, [vp, P(i32)])
    _sig(L, "fs_ctx_set_option", C.c_int, [vp, C.c_char_p, i64])
    _sig(L, "fs_map_new", C.c_int, [vp, P(vp), vp, vp, i64, i64])
    _sig(L, "fs_map_new_i32", C.c_int, [vp, P(vp), vp, vp, i64, i64])
    _sig(L, "fs_map_wrap_device", C.c_int, [vp, P(vp), vp, vp, i64, i64])
    _sig(L, "fs_map_free", C.c_int, [vp, vp])
    _sig(L, "fs_map_shape", C.c_int, [vp, P(i64), P(i64)])
    _sig(L, "fs_map_quads_dev", vp, [vp])
    _sig(L, "fs_map_colors_dev", vp, [vp])
    _sig(L, "fs_num_depths", i32, [f32, P(Params)])
    _sig(L, "fs_render_device", C.c_int, [vp, vp, P(Camera), P(Params), i32, i32, vp])
    _sig(L, "fs_render", C.c_int, [vp, vp, P(Camera), P(Params), i32, i32, vp])
    _sig(L, "fs_plan_new", C.c_int, [vp, P(vp), P(vp), i32, P(Params), P(View), i32])
    _sig(L, "fs_plan_free", None, [vp])
    _sig(L, "fs_plan_set_cameras", C.c_int, [vp, P(Camera), i32])
    _sig(L, "fs_plan_run", C.c_int, [vp])
    _sig(L, "fs_plan_run_per_view", C.c_int, [vp])
    _sig(L, "fs_plan_kernel_ms", C.c_int, [vp, P(f32)])
    _sig(L, "fs_plan_frame_dev", vp, [vp, i32])
    _sig(L, "fs_plan_frame_offset", i64, [vp, i32])
    _sig(L, "fs_plan_total_pixels", i64, [vp])
    _sig(L, "fs_plan_download", C.c_int, [vp, vp])
    _sig(L, "fs_plan_run_download", C.c_int, [vp, vp, i32])
    _sig(L, "fs_plan_download_bytes", C.c_int, [vp, P(i64), P(i64)])
    _sig(L, "fs_plan_get_tune", C.c_int, [vp, P(i32)])
    _sig(L, "fs_plan_set_tune", C.c_int, [vp, P(i32)])
    _sig(L, "fs_plan_signature", C.c_int, [vp, P(i64)])
    _sig(L, "fs_autotune_frame", C.c_int,
         [vp, vp, P(Camera), P(Params), i32, i32, i32, P(i32), P(f32)])
    _sig(L, "fs_plan_autotune", C.c_int, [vp, i32, P(i32), P(f32)])
    _sig(L, "fs_tune_count", C.c_int, [])
    _sig(L, "fs_tune_get", C.c_int, [C.c_int, P(i32)])
    _sig(L, "fs_host_alloc", vp, [C.c_size_t])
    _sig(L, "fs_host_free", None, [vp])
    _sig(L, "fs_server_new", C.c_int, [vp, P(vp), P(vp), i32, P(Params), P(ServerConfig)])
    _sig(L, "fs_server_free", None, [vp])
    _sig(L, "fs_server_run", C.c_int, [vp, P(Request), i32, i32, P(ServeStats)])
    _sig(L, "fsgen_heights", C.c_int, [u64, i32, f32, vp])
    _sig(L, "fsgen_colors", C.c_int, [u64, vp, i64, i32, vp])
    _sig(L, "fsgen_local_max", i32, [vp, i32, i32, f32, f32])
    _sig(L, "fsgen_cameras", C.c_int,
         [u64, vp, i32, i32, i32, f32, f32, f32, f32, i32, P(Camera)])
    _sig(L, "fsgen_walk", C.c_int,
         [u64, vp, i32, i32, i32, f32, f32, f32, f32, f32, i32, P(Camera)])
    _sig(L, "fs_png_read", C.c_int, [C.c_char_p, P(vp), P(i64), P(i64)])
    _sig(L, "fs_png_decode", C.c_int, [vp, C.c_size_t, P(vp), P(i64), P(i64)])
    _sig(L, "fs_png_write", C.c_int, [C.c_char_p, vp, i64, i64])
    _sig(L, "fs_data_read", C.c_int, [C.c_char_p, P(vp), C.c_char_p, P(i32), P(i64)])
    _sig(L, "fs_data_write", C.c_int, [C.c_char_p, vp, C.c_char_p, i32, P(i64)])
    _sig(L, "fs_free", None, [vp])
    _sig(L, "fs_map_load_png", C.c_int, [vp, P(vp), C.c_char_p, C.c_char_p])
    _LIB = L
    return L


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return int(a)


def default_params(**kw) -> Params:
    p = lib().fs_params_default()
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def num_depths(distance: float, params: Params | None = None) -> int:
    return lib().fs_num_depths(float(distance), C.byref(params or default_params()))


# ---- synthetic inputs -----------------------------------------------------------------

def _check(rc: int, what: str):
    if rc != 0:
        raise FsError(rc, what)


def gen_heights(seed: int, size: int, roughness: float = 0.55) -> np.ndarray:
    out = np.empty((size, size), np.uint8)
    _check(lib().fsgen_heights(seed, size, roughness, _ptr(out)), "fsgen_heights")
    return out


def gen_colors(seed: int, heights: np.ndarray, noise: int = 12) -> np.ndarray:
    h = np.ascontiguousarray(heights, np.uint8)
    out = np.empty(h.shape, np.uint32)
    _check(lib().fsgen_colors(seed, _ptr(h), h.size, noise, _ptr(out)), "fsgen_colors")
    return out


def local_max(heights: np.ndarray, x: float, y: float) -> int:
    h = np.ascontiguousarray(heights, np.uint8)
    return lib().fsgen_local_max(_ptr(h), h.shape[0], h.shape[1], x, y)


def gen_cameras(seed: int, heights: np.ndarray, count: int, above=(40.0, 40.0),
                distance=(800.0, 800.0), screen_h: int = 240) -> list[Camera]:
    h = np.ascontiguousarray(heights, np.uint8)
    arr = (Camera * count)()
    _check(lib().fsgen_cameras(seed, _ptr(h), h.shape[0], h.shape[1], count, above[0], above[1],
                               distance[0], distance[1], screen_h, arr), "fsgen_cameras")
    return list(arr)


# ---- map ingest and frame output (PNG, Futhark binary data format) ------------

_DATA_TYPES = {" i32": np.int32, " u32": np.uint32, "  u8": np.uint8, "  i8": np.int8,
               " f32": np.float32, " i16": np.int16, " u16": np.uint16, " i64": np.int64,
               " u64": np.uint64, " f64": np.float64, "bool": np.bool_}


def _take_u32(p, rows, cols) -> np.ndarray:
    try:
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint32)),
                                     shape=(rows, cols)).copy()
    finally:
        lib().fs_free(p)


def png_read(path) -> np.ndarray:
    """fs_png_read: a PNG as [rows][cols] u32 0xFFRRGGBB words."""
    p, r, c = C.c_void_p(), C.c_int64(), C.c_int64()
    _check(lib().fs_png_read(str(path).encode(), C.byref(p), C.byref(r), C.byref(c)),
           f"fs_png_read({path})")
    return _take_u32(p, r.value, c.value)


def png_decode(data: bytes) -> np.ndarray:
    buf = C.create_string_buffer(bytes(data), len(data))
    p, r, c = C.c_void_p(), C.c_int64(), C.c_int64()
    _check(lib().fs_png_decode(buf, len(data), C.byref(p), C.byref(r), C.byref(c)),
           "fs_png_decode")
    return _take_u32(p, r.value, c.value)


def png_write(path, argb: np.ndarray):
    a = np.ascontiguousarray(argb, np.uint32)
    assert a.ndim == 2
    _check(lib().fs_png_write(str(path).encode(), _ptr(a), a.shape[0], a.shape[1]),
           f"fs_png_write({path})")


def data_read(path) -> np.ndarray:
    """fs_data_read: a value in the Futhark binary data format."""
    p, t, r = C.c_void_p(), C.create_string_buffer(5), C.c_int32()
    dims = (C.c_int64 * 8)()
    _check(lib().fs_data_read(str(path).encode(), C.byref(p), t, C.byref(r), dims),
           f"fs_data_read({path})")
    try:
        dt = np.dtype(_DATA_TYPES[t.value.decode()])
        shape = tuple(dims[i] for i in range(r.value))
        n = int(np.prod(shape)) if shape else 1
        raw = C.string_at(p, n * dt.itemsize) if n else b""
        return np.frombuffer(raw, dt).reshape(shape).copy()
    finally:
        lib().fs_free(p)


def data_write(path, array: np.ndarray, type_name: str | None = None):
    a = np.ascontiguousarray(array)
    if type_name is None:
        type_name = {np.dtype(v): k for k, v in _DATA_TYPES.items()}[a.dtype]
    dims = (C.c_int64 * max(1, a.ndim))(*a.shape)
    _check(lib().fs_data_write(str(path).encode(), _ptr(a), type_name.encode(), a.ndim, dims),
           f"fs_data_write({path})")


def gen_walk(seed: int, heights: np.ndarray, count: int, step: float = 2.0, yaw: float = 0.02,
             above=(30.0, 120.0), distance: float = 3000.0, screen_h: int = 1080) -> list[Camera]:
    h = np.ascontiguousarray(heights, np.uint8)
    arr = (Camera * count)()
    _check(lib().fsgen_walk(seed, _ptr(h), h.shape[0], h.shape[1], count, step, yaw, above[0],
                            above[1], distance, screen_h, arr), "fsgen_walk")
    return list(arr)


# ---- objects ---------------------------------------------------------------------------

class Context:
    """fs_ctx: one device, one stream, error text, scratch buffers."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().fs_ctx_new(C.byref(self._h), device)
        if rc != 0:
            msg = self.error() if self._h else "fs_ctx_new"
            if self._h:
                lib().fs_ctx_free(self._h)
                self._h = C.c_void_p()
            raise FsError(rc, msg or "fs_ctx_new")
        # maps, plans and servers made on this context: closed before it
        self._deps: "weakref.WeakSet" = weakref.WeakSet()
        _LIVE.add(self)

    @property
    def handle(self):
        return self._h

    def error(self) -> str:
        p = lib().fs_ctx_get_error(self._h)
        if not p:
            return ""
        s = C.string_at(p).decode()
        C.CDLL(None).free(C.c_void_p(p))
        return s

    def check(self, rc: int, what: str):
        if rc != 0:
            raise FsError(rc, f"{what}: {self.error()}")

    def sync(self):
        self.check(lib().fs_ctx_sync(self._h), "sync")

    def set_stream(self, stream_handle: int | None):
        self.check(lib().fs_ctx_set_stream(self._h, stream_handle or None), "set_stream")

    @property
    def stream_handle(self) -> int:
        """The cudaStream_t every asynchronous call of this context uses."""
        return lib().fs_ctx_get_stream(self._h) or 0

    @property
    def launches(self) -> int:
        return lib().fs_ctx_kernel_launches(self._h)

    def set_option(self, name: str, value: int):
        self.check(lib().fs_ctx_set_option(self._h, name.encode(), int(value)), "set_option")

    def force_tune(self, tune=None):
        """tune = (tile_width, lanes_per_column, depth_per_lane, stage) or None."""
        t = (C.c_int32 * 5)(*(tuple(tune) + (0,) * (5 - len(tune)))) if tune else None
        self.check(lib().fs_ctx_force_tune(self._h, t), "force_tune")

    def kernel_ms(self) -> float:
        """Device time of the kernels of the last plain call made with option "time"."""
        ms = C.c_float()
        self.check(lib().fs_ctx_kernel_ms(self._h, C.byref(ms)), "kernel_ms")
        return ms.value

    def measure_l2_read_gbs(self, nbytes: int = 48 << 20, reps: int = 40) -> float:
        """L2 read bandwidth (GB/s) of an L2-resident buffer (a roofline denominator)."""
        gbs = C.c_float()
        self.check(lib().fs_measure_l2_read_gbs(self._h, nbytes, reps, C.byref(gbs)), "l2 probe")
        return gbs.value

    def stats(self, enable: bool = True):
        out = (C.c_uint64 * 2)()
        self.check(lib().fs_ctx_stats(self._h, int(enable), out), "stats")
        return int(out[0]), int(out[1])

    def close(self):
        """Frees the context after the servers, plans and maps made on it."""
        if self._h:
            deps = list(self._deps)
            for kind in (Server, Plan, Map):
                for o in deps:
                    if isinstance(o, kind):
                        o.close()
            lib().fs_ctx_free(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self, _fin=sys.is_finalizing):
        # the default binds the check at class creation: module globals may
        # already be gone when a late collection runs this
        if _fin():
            return
        try:
            self.close()
        except Exception:
            pass

    # -- renders --
    def render(self, fmap: "Map", cam: Camera, width: int, height: int,
               params: Params | None = None, out: np.ndarray | None = None) -> np.ndarray:
        """Plain per-frame render into host memory ([height][width] u32 ARGB)."""
        if out is None:
            out = np.empty((height, width), np.uint32)
        assert out.dtype == np.uint32 and out.flags.c_contiguous and out.size == width * height
        self.check(lib().fs_render(self._h, fmap.handle, C.byref(cam),
                                   C.byref(params or default_params()), width, height, _ptr(out)),
                   "fs_render")
        return out

    def render_device(self, fmap: "Map", cam: Camera, width: int, height: int, out_dev,
                      params: Params | None = None):
        """Asynchronous render into device memory (pointer or tensor with data_ptr)."""
        self.check(lib().fs_render_device(self._h, fmap.handle, C.byref(cam),
                                          C.byref(params or default_params()), width, height,
                                          _ptr(out_dev)), "fs_render_device")

    def autotune_frame(self, fmap: "Map", cam: Camera, width: int, height: int,
                       params: Params | None = None, reps: int = 5):
        out = (C.c_int32 * 5)()
        ms = C.c_float()
        self.check(lib().fs_autotune_frame(self._h, fmap.handle, C.byref(cam),
                                           C.byref(params or default_params()), width, height,
                                           reps, out, C.byref(ms)), "autotune_frame")
        return tuple(out[:4]), ms.value


class Map:
    """fs_map: a resident height/colour map pair."""

    def __init__(self, ctx: Context, heights: np.ndarray, colors: np.ndarray):
        self.ctx = ctx
        self._h = C.c_void_p()
        assert heights.shape == colors.shape and heights.ndim == 2
        if heights.dtype == np.int32:
            h = np.ascontiguousarray(heights)
            fn = lib().fs_map_new_i32
        else:
            h = np.ascontiguousarray(heights, np.uint8)
            fn = lib().fs_map_new
        c = np.ascontiguousarray(colors, np.uint32)
        ctx.check(fn(ctx.handle, C.byref(self._h), _ptr(h), _ptr(c), h.shape[0], h.shape[1]),
                  "fs_map_new")
        self.shape = h.shape
        ctx._deps.add(self)
        _LIVE.add(self)

    @classmethod
    def from_png(cls, ctx: Context, color_png, height_png) -> "Map":
        """fs_map_load_png: colour and height images as c/interactive.c loads them."""
        m = cls.__new__(cls)
        m.ctx = ctx
        m._h = C.c_void_p()
        ctx.check(lib().fs_map_load_png(ctx.handle, C.byref(m._h), str(color_png).encode(),
                                        str(height_png).encode()), "fs_map_load_png")
        r, c = C.c_int64(), C.c_int64()
        lib().fs_map_shape(m._h, C.byref(r), C.byref(c))
        m.shape = (r.value, c.value)
        ctx._deps.add(m)
        _LIVE.add(m)
        return m

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().fs_map_free(self.ctx.handle, self._h)
            self._h = C.c_void_p()

    def __del__(self, _fin=sys.is_finalizing):
        # the default binds the check at class creation: module globals may
        # already be gone when a late collection runs this
        if _fin():
            return
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """fs_plan: batched multi-view render (persistent kernel, CUDA graph)."""

    def __init__(self, ctx: Context, maps: Sequence[Map], views: Sequence[tuple],
                 params: Params | None = None):
        """views: (Camera, width, height[, map_index]) tuples."""
        self.ctx = ctx
        self._h = C.c_void_p()
        arr = (View * len(views))()
        for i, v in enumerate(views):
            arr[i].cam = v[0]
            arr[i].width = v[1]
            arr[i].height = v[2]
            arr[i].map = v[3] if len(v) > 3 else 0
        mp = (C.c_void_p * len(maps))(*[m.handle.value for m in maps])
        self.params = params or default_params()
        ctx.check(lib().fs_plan_new(ctx.handle, C.byref(self._h), mp, len(maps),
                                    C.byref(self.params), arr, len(views)), "fs_plan_new")
        self.sizes = [(v[1], v[2]) for v in views]
        self.nviews = len(views)
        ctx._deps.add(self)
        _LIVE.add(self)

    @property
    def handle(self):
        return self._h

    def run(self):
        self.ctx.check(lib().fs_plan_run(self._h), "fs_plan_run")

    def run_per_view(self):
        self.ctx.check(lib().fs_plan_run_per_view(self._h), "fs_plan_run_per_view")

    def kernel_ms(self) -> float:
        """Device time of the render kernel in the last run (waits for it)."""
        ms = C.c_float()
        self.ctx.check(lib().fs_plan_kernel_ms(self._h, C.byref(ms)), "fs_plan_kernel_ms")
        return ms.value

    def set_cameras(self, cams: Iterable[Camera]):
        cams = list(cams)
        arr = (Camera * len(cams))(*cams)
        self.ctx.check(lib().fs_plan_set_cameras(self._h, arr, len(cams)), "set_cameras")

    @property
    def total_pixels(self) -> int:
        return lib().fs_plan_total_pixels(self._h)

    def frame_offset(self, i: int) -> int:
        return lib().fs_plan_frame_offset(self._h, i)

    def frame_dev(self, i: int) -> int:
        return lib().fs_plan_frame_dev(self._h, i)

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.total_pixels, np.uint32)
        self.ctx.check(lib().fs_plan_download(self._h, _ptr(out)), "fs_plan_download")
        return out

    def run_download(self, out: np.ndarray | None = None, groups: int = 4) -> np.ndarray:
        """fs_plan_run_download: render and copy frames to the host, overlapped."""
        if out is None:
            out = np.empty(self.total_pixels, np.uint32)
        self.ctx.check(lib().fs_plan_run_download(self._h, _ptr(out), groups),
                       "fs_plan_run_download")
        return out

    def download_bytes(self) -> tuple[int, int]:
        """(bytes copied device to host, bytes of sky rows written on the host) of
        the last run_download."""
        copied, filled = C.c_int64(), C.c_int64()
        self.ctx.check(lib().fs_plan_download_bytes(self._h, C.byref(copied), C.byref(filled)),
                       "fs_plan_download_bytes")
        return copied.value, filled.value

    def frames(self, flat: np.ndarray | None = None) -> list[np.ndarray]:
        flat = self.download() if flat is None else flat
        res = []
        for i, (w, h) in enumerate(self.sizes):
            o = self.frame_offset(i)
            res.append(flat[o:o + w * h].reshape(h, w))
        return res

    def get_tune(self):
        """(tile_width, lanes_per_column, depth_per_lane, stage, persistent_ctas)"""
        out = (C.c_int32 * 5)()
        self.ctx.check(lib().fs_plan_get_tune(self._h, out), "get_tune")
        return tuple(out)

    def set_tune(self, tw: int, lc: int, u: int, stage: int = 1, ctas: int = 0):
        t = (C.c_int32 * 5)(tw, lc, u, stage, ctas)
        self.ctx.check(lib().fs_plan_set_tune(self._h, t), "set_tune")

    def autotune(self, reps: int = 3):
        out = (C.c_int32 * 5)()
        ms = C.c_float()
        self.ctx.check(lib().fs_plan_autotune(self._h, reps, out, C.byref(ms)), "autotune")
        return tuple(out), ms.value

    def close(self):
        if self._h:
            lib().fs_plan_free(self._h)
            self._h = C.c_void_p()

    def __del__(self, _fin=sys.is_finalizing):
        # the default binds the check at class creation: module globals may
        # already be gone when a late collection runs this
        if _fin():
            return
        try:
            self.close()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host memory viewed as a numpy array (fs_host_alloc)."""

    def __init__(self, shape, dtype=np.uint32):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self._p = lib().fs_host_alloc(nbytes)
        if not self._p:
            raise FsError(4, "fs_host_alloc")
        self.array = np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(self._p))
        self.array = self.array.view(dtype).reshape(shape)
        _LIVE.add(self)

    @property
    def ptr(self) -> int:
        return self._p

    def close(self):
        if self._p:
            self.array = None
            lib().fs_host_free(self._p)
            self._p = None

    def __del__(self, _fin=sys.is_finalizing):
        # the default binds the check at class creation: module globals may
        # already be gone when a late collection runs this
        if _fin():
            return
        try:
            self.close()
        except Exception:
            pass


class Server:
    """fs_server: continuous-batching request loop over the persistent kernel."""

    def __init__(self, ctx: Context, maps: Sequence[Map], budget_bytes: int, nsessions: int,
                 max_batch: int = 64, slots: int = 3, max_distance: float = 3000.0,
                 tune=None, params: Params | None = None):
        self.ctx = ctx
        self._h = C.c_void_p()
        self.params = params or default_params()
        cfg = ServerConfig(budget_bytes, nsessions, max_batch, slots,
                           num_depths(max_distance, self.params))
        for i, v in enumerate(tuple(tune or ()) + (0,) * (5 - len(tuple(tune or ())))):
            cfg.tune[i] = v
        mp = (C.c_void_p * len(maps))(*[m.handle.value for m in maps])
        ctx.check(lib().fs_server_new(ctx.handle, C.byref(self._h), mp, len(maps),
                                      C.byref(self.params), C.byref(cfg)), "fs_server_new")
        ctx._deps.add(self)
        _LIVE.add(self)

    def run(self, requests, realtime: bool = False) -> dict:
        st = ServeStats()
        self.ctx.check(lib().fs_server_run(self._h, requests, len(requests), int(realtime),
                                           C.byref(st)), "fs_server_run")
        return st.as_dict()

    def close(self):
        if self._h:
            lib().fs_server_free(self._h)
            self._h = C.c_void_p()

    def __del__(self, _fin=sys.is_finalizing):
        # the default binds the check at class creation: module globals may
        # already be gone when a late collection runs this
        if _fin():
            return
        try:
            self.close()
        except Exception:
            pass


def tune_table() -> list[tuple[int, int, int, int]]:
    """Compiled kernel configurations (tile_width, lanes_per_column, depth_per_lane, stage)."""
    L = lib()
    out = []
    for i in range(L.fs_tune_count()):
        t = (C.c_int32 * 5)()
        L.fs_tune_get(i, t)
        out.append(tuple(t[:4]))
    return out
