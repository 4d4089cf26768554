"""The C-ABI library: loads, exports every function the public headers declare,
and its host-side logic (parameters, depth counts, generators, errors) works
without a GPU."""
import ctypes as C
import hashlib
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
KAT_N = {400.0: 894, 800.0: 1265, 1000.0: 1414, 1600.0: 1789, 2000.0: 2000, 3000.0: 2449,
         6000.0: 3464}


def declared_functions(header: Path) -> list[str]:
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = "\n".join(l for l in text.splitlines() if not l.lstrip().startswith("#"))
    names = re.findall(r"\b([A-Za-z_]\w*)\s*\([^;{}]*\)\s*;", text)
    return sorted({n for n in names if n not in ("sizeof",)})


@pytest.mark.parametrize("header", sorted((ROOT / "include").glob("*.h")), ids=lambda p: p.name)
def test_exports_every_declared_symbol(fs, header):
    lib = C.CDLL(str(fs.library_path()))
    names = declared_functions(header)
    assert names, f"no declarations parsed from {header}"
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"{header.name}: not exported: {missing}"


def test_params_default(fs):
    p = fs.default_params()
    assert (p.invz_param1, p.invz_param2, p.magic_number) == (np.float32(0.001), 0.0, 0.0)
    assert (p.height_filter, p.color_filter, p.gap_rule, p.floor_n) == (1, 1, 0, 1)


@pytest.mark.parametrize("D,n", sorted(KAT_N.items()))
def test_num_depths_kat(fs, D, n):
    assert fs.num_depths(D) == n


def test_num_depths_mode_b(fs):
    p = fs.default_params(invz_param1=0.005, invz_param2=1.0, floor_n=0)
    assert fs.num_depths(800.0, p) == 400


def test_generators_are_deterministic(fs):
    """Fixed seeds give fixed bytes on every host (the digests are committed)."""
    hm = fs.gen_heights(7, 256, 0.55)
    cm = fs.gen_colors(8, hm, 12)
    assert hm.min() == 0 and hm.max() == 255
    assert np.all((cm >> 24) == 0xFF)
    assert np.array_equal(hm, fs.gen_heights(7, 256, 0.55))
    golden = (ROOT / "tests" / "golden" / "generators.txt").read_text().split()
    assert hashlib.sha256(hm.tobytes()).hexdigest() == golden[0]
    assert hashlib.sha256(cm.tobytes()).hexdigest() == golden[1]
    cams = fs.gen_cameras(9, hm, 4, above=(20, 200), distance=(400, 3000), screen_h=240)
    walk = fs.gen_walk(10, hm, 8, distance=3000.0, screen_h=1080)
    blob = b"".join(bytes(c) for c in cams + walk)
    assert hashlib.sha256(blob).hexdigest() == golden[2]


def test_camera_generator_semantics(fs):
    hm = fs.gen_heights(7, 256, 0.55)
    for c in fs.gen_cameras(11, hm, 16, above=(20, 200), distance=(400, 3000), screen_h=480):
        above = c.height - fs.local_max(hm, c.x, c.y)
        assert 20 - 1e-3 <= above <= 200 + 1e-3
        assert 400 <= c.distance <= 3000 and 0 <= c.angle < 6.2832
        assert c.horizon == 240 and abs(c.fov - 1.2) < 1e-6
    walk = fs.gen_walk(12, hm, 64, step=2.0, yaw=0.02, distance=3000.0, screen_h=1080)
    for a, b in zip(walk, walk[1:]):
        assert abs(b.angle - a.angle) <= 0.02 + 1e-6
        assert abs(np.hypot(b.x - a.x, b.y - a.y) - 2.0) < 1e-3
        assert 30 - 1e-3 <= b.height - fs.local_max(hm, b.x, b.y) <= 120 + 1e-3


def test_errors_without_device_or_with_bad_args(fs):
    L = fs.lib()
    # NULL context / NULL arguments are rejected, never dereferenced
    assert L.fs_render(None, None, None, None, 16, 16, None) == 1
    assert L.fs_render_device(None, None, None, None, 16, 16, None) == 1
    assert L.fs_ctx_sync(None) == 1
    try:
        ctx = fs.Context(0)
    except fs.FsError as e:
        assert e.code == 2  # FS_ERR_CUDA: no device in this environment
        return
    with ctx:
        hm = fs.gen_heights(1, 64)
        fmap = fs.Map(ctx, hm, fs.gen_colors(2, hm))
        cam = fs.gen_cameras(3, hm, 1)[0]
        with pytest.raises(fs.FsError) as ei:
            ctx.render(fmap, cam, 16, 20000)  # taller than the supported maximum
        assert ei.value.code == 1
        bad = fs.Camera(*cam.as_tuple())
        bad.distance = -100.0
        with pytest.raises(fs.FsError) as ei:
            ctx.render(fmap, bad, 16, 16)
        assert ei.value.code == 3  # empty depth range


def test_tune_table(fs):
    t = fs.tune_table()
    assert len(t) >= 8 and all(len(x) == 4 for x in t)
    assert any(x[3] == 1 for x in t) and any(x[3] == 0 for x in t)



def test_context_close_closes_its_objects(fs, monkeypatch):
    """Closing a context first closes the servers, plans and maps made on it
    (their handles refer to the context), then frees the context."""
    import weakref

    order = []
    monkeypatch.setattr(fs.Server, "close", lambda self: order.append("server"))
    monkeypatch.setattr(fs.Plan, "close", lambda self: order.append("plan"))
    monkeypatch.setattr(fs.Map, "close", lambda self: order.append("map"))

    class FakeLib:
        def fs_ctx_free(self, h):
            order.append("context")

    monkeypatch.setattr(fs, "lib", lambda: FakeLib())
    ctx = fs.Context.__new__(fs.Context)
    ctx._h = C.c_void_p(1)
    ctx._deps = weakref.WeakSet()
    objs = [fs.Map.__new__(fs.Map), fs.Plan.__new__(fs.Plan), fs.Server.__new__(fs.Server)]
    for o in objs:
        ctx._deps.add(o)
    ctx.close()
    assert order == ["server", "plan", "map", "context"]
    assert not ctx._h
    ctx.close()  # a second close does nothing
    assert order == ["server", "plan", "map", "context"]
