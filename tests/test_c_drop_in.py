"""The drop-in header from C: tests/c/drop_in.c includes include/libfutspace.h
and makes the reference host program's calls (c/interactive.c:25-71,99) with
that program's own types, so a C compiler checks the header's names,
const-ness and pointer types the way c/interactive.c would see them. The CPU
test compiles and links it with every warning an error; the GPU test runs it
and diffs its frame against the oracle."""
import subprocess

import numpy as np
import pytest

from conftest import ROOT, count_diff

SRC = ROOT / "tests" / "c" / "drop_in.c"


def _compile(fs, out_dir):
    exe = out_dir / "drop_in"
    lib = fs.library_path()
    cmd = ["gcc", "-std=c99", "-O1", "-Wall", "-Wextra", "-Werror", "-pedantic",
           "-I", str(ROOT / "include"), str(SRC), "-o", str(exe),
           "-L", str(lib.parent), "-l" + lib.stem[3:], f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_drop_in_header_compiles_from_c(fs, tmp_path):
    exe = _compile(fs, tmp_path)
    assert exe.exists()
    # the header alone, as a C++ translation unit too (lys is C, some hosts are C++)
    cpp = tmp_path / "h.cc"
    cpp.write_text('#include "libfutspace.h"\nint main() { return 0; }\n')
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I",
                        str(ROOT / "include"), "-c", str(cpp), "-o", str(tmp_path / "h.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_drop_in_program_renders_like_the_oracle(fs, orc, tmp_path):
    from test_gpu_compat import sun_vector
    exe = _compile(fs, tmp_path)
    hm = fs.gen_heights(41, 256, 0.55)
    cm = fs.gen_colors(42, hm, 12)
    hi = hm.astype(np.int32) | np.int32(0x3C00)  # update_map keeps the low byte
    cm.astype("<u4").tofile(tmp_path / "c.raw")
    hi.astype("<i4").tofile(tmp_path / "h.raw")
    r = subprocess.run([str(exe), str(tmp_path / "c.raw"), str(tmp_path / "h.raw"), "256", "256",
                        str(tmp_path / "out.raw")], capture_output=True, text=True, timeout=300)
    if r.returncode != 0 and "no CUDA" in r.stderr:
        pytest.skip(r.stderr)
    assert r.returncode == 0, r.stderr
    raw = (tmp_path / "out.raw").read_bytes()
    text = np.frombuffer(raw[:36], "<f4")
    dims = np.frombuffer(raw[36:52], "<i8")
    frame = np.frombuffer(raw[52:], "<u4").reshape(int(dims[0]), int(dims[1]))
    assert tuple(dims) == (120, 160)
    x, y, ang, height, hor, dist, sun_h, sun_a, fov = (float(v) for v in text)
    # the shadow map update_map precomputed from the initial sun (0.1, 0.1)
    shadow = orc.shadowmap(hm, cm, sun_vector(0.1, 0.1), threads=0)
    sky = orc.lib().fso_scale(0xFF9090E0, sun_h)
    cam = dict(x=x, y=y, height=height, angle=ang, horizon=hor, distance=dist, fov=fov,
               sky_color=sky)
    want = orc.render(cam, orc.make_params(), hm, shadow, 160, 120, threads=0)
    assert count_diff(frame, want) == 0
