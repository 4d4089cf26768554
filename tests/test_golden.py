"""Known-answer frames (tests/golden, made by tests/golden/make_golden.py from
the oracle): the oracle reproduces them on this host, and the CUDA path
reproduces them on the GPU."""
import ctypes as C
import hashlib
import json
import struct
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

_libm = C.CDLL("libm.so.6")
for _n in ("sinf", "cosf"):
    getattr(_libm, _n).restype = C.c_float
    getattr(_libm, _n).argtypes = [C.c_float]


def _cases():
    return json.loads((GOLDEN / "frames.json").read_text())


def _check_libm(c):
    ang = np.float32(c["cam"][3])
    bits = lambda v: struct.unpack("<I", struct.pack("<f", v))[0]  # noqa: E731
    if (bits(_libm.sinf(ang)), bits(_libm.cosf(ang))) != (c["sin_bits"], c["cos_bits"]):
        pytest.fail("this host's sinf/cosf round differently from the fixture's host: "
                    "frames are not comparable")


def _frame_ok(c, frame, full):
    if c["full"]:
        assert np.array_equal(frame, full[f"f{_cases().index(c)}"])
    assert hashlib.sha256(np.ascontiguousarray(frame).tobytes()).hexdigest() == c["sha256"]


def test_oracle_reproduces_golden(fs, orc):
    import make_golden
    full = np.load(GOLDEN / "frames.npz")
    for c in _cases():
        _check_libm(c)
        frame, _, _ = make_golden.render_case(c)
        _frame_ok(c, frame, full)


@pytest.mark.gpu
def test_gpu_reproduces_golden(fs, orc, gpu_ctx):
    import make_golden
    full = np.load(GOLDEN / "frames.npz")
    for c in _cases():
        _check_libm(c)
        hm, cm = make_golden.maps(*c["map"])
        fmap = fs.Map(gpu_ctx, hm, cm)
        d, z0, scale, hf, cf, gap, floor_n = c["params"]
        p = fs.default_params(invz_param1=d, invz_param2=z0, magic_number=scale,
                              height_filter=hf, color_filter=cf, gap_rule=gap, floor_n=floor_n)
        frame = gpu_ctx.render(fmap, fs.Camera(*c["cam"]), c["W"], c["H"], params=p)
        _frame_ok(c, frame, full)
        fmap.close()
