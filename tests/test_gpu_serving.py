"""Serving (continuous batching): every frame is the same rendered alone, in a
mix of concurrent requests and under Poisson arrivals, and equals the oracle.
Bit-exact (u32 frames, no tolerance)."""
import numpy as np
import pytest

from conftest import count_diff

pytestmark = pytest.mark.gpu

SIZES = [(320, 240), (640, 480), (257, 131), (128, 96)]


def _requests(fs, maps_np, nsess, per_sess, seed):
    """per_sess consecutive walk frames for each session; session s uses map s % 2."""
    rng = np.random.default_rng(seed)
    reqs = []
    for s in range(nsess):
        hm = maps_np[s % 2][0]
        w, h = SIZES[int(rng.integers(0, len(SIZES)))]
        walk = fs.gen_walk(seed * 100 + s, hm, per_sess, step=2.0, yaw=0.05, above=(20, 120),
                           distance=float(rng.uniform(300, 1200)), screen_h=h)
        for cam in walk:
            reqs.append((s, s % 2, w, h, cam))
    return reqs


def _fill(fs, specs, bufs, arrivals=None):
    arr = (fs.Request * len(specs))()
    for i, (s, m, w, h, cam) in enumerate(specs):
        r = arr[i]
        r.session, r.map, r.width, r.height, r.cam = s, m, w, h, cam
        r.host_out = bufs[i].ptr
        r.arrival_ns = 0 if arrivals is None else int(arrivals[i])
    return arr


@pytest.mark.parametrize("tune", [None, (128, 1, 4, 0), (8, 64, 8, 2)],
                         ids=["default", "direct", "cooperative"])
def test_alone_equals_mix_equals_oracle(fs, orc, gpu_ctx, maps1024, maps256, tune):
    """The default server (cooperative tile per launch where the tallest frame
    fits, else direct painting) and each form alone."""
    maps_np = [maps1024, maps256]
    fmaps = [fs.Map(gpu_ctx, h, c) for h, c in maps_np]
    specs = _requests(fs, maps_np, nsess=8, per_sess=4, seed=5)
    bufs = [fs.PinnedBuffer((h, w)) for (_, _, w, h, _) in specs]
    srv = fs.Server(gpu_ctx, fmaps, budget_bytes=16 << 20, nsessions=8, max_batch=8, slots=3,
                    max_distance=1200.0, tune=tune)
    try:
        # in the mix: everything released at once (admission + batching decide)
        reqs = _fill(fs, specs, bufs)
        st = srv.run(reqs)
        assert st["errors"] == 0 and st["requests"] == len(specs)
        assert st["batches"] >= 2 and st["max_inflight"] >= 2
        mixed = [b.array.copy() for b in bufs]
        # per session the frames complete in order (one request in flight per session)
        for s in range(8):
            done = [reqs[i].done_ns for i, sp in enumerate(specs) if sp[0] == s]
            assert done == sorted(done)
        # alone: one request per run
        for i, sp in enumerate(specs):
            b = bufs[i]
            b.array[:] = 0
            one = _fill(fs, [sp], [b])
            srv.run(one)
            assert one[0].status == 0
            assert count_diff(b.array, mixed[i]) == 0, i
        # Poisson arrivals, paced on the host clock
        rng = np.random.default_rng(9)
        arrivals = np.cumsum(rng.exponential(1e9 / 4000.0, len(specs)))
        for b in bufs:
            b.array[:] = 0
        reqs = _fill(fs, specs, bufs, arrivals)
        st = srv.run(reqs, realtime=True)
        assert st["errors"] == 0 and st["p99_ms"] >= st["p50_ms"] > 0
        for i in range(len(specs)):
            assert count_diff(bufs[i].array, mixed[i]) == 0, i
        # oracle on a sample
        p = fs.default_params()
        for i in range(0, len(specs), 5):
            s, m, w, h, cam = specs[i]
            hm, cm = maps_np[m]
            ref = orc.render(cam, orc.params_from(p), hm, cm, w, h, threads=0)
            assert count_diff(mixed[i], ref) == 0, i
    finally:
        srv.close()
        for b in bufs:
            b.close()


def test_budget_admission(fs, gpu_ctx, maps256):
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    cams = fs.gen_cameras(3, hm, 6, above=(20, 80), distance=(200, 400), screen_h=240)
    # room for two 320x240 frames only; a 640x480 frame can never fit
    srv = fs.Server(gpu_ctx, [fmap], budget_bytes=2 * 320 * 240 * 4 + 512, nsessions=8,
                    max_batch=8, slots=2, max_distance=400.0)
    bufs = [fs.PinnedBuffer((240, 320)) for _ in range(6)] + [fs.PinnedBuffer((480, 640))]
    try:
        specs = [(i, 0, 320, 240, c) for i, c in enumerate(cams)] + [(6, 0, 640, 480, cams[0])]
        reqs = _fill(fs, specs, bufs)
        st = srv.run(reqs)
        assert [r.status for r in reqs] == [0] * 6 + [5]  # FS_ERR_BUDGET for the big one
        assert st["max_inflight"] <= 2 and st["peak_arena_bytes"] <= 2 * 320 * 240 * 4 + 512
        ref = [b.array.copy() for b in bufs[:6]]
        for i in range(6):
            one = _fill(fs, [specs[i]], [bufs[i]])
            srv.run(one)
            assert count_diff(bufs[i].array, ref[i]) == 0
    finally:
        srv.close()
        for b in bufs:
            b.close()


@pytest.mark.parametrize("mode", ["smoothing", "effects"])
def test_serving_modes(fs, orc, gpu_ctx, maps256, mode):
    """A server built with the smoothing branch or the shading/fog epilogue
    renders every request as the oracle does in that mode, alone or mixed."""
    hm, cm = maps256
    fmap = fs.Map(gpu_ctx, hm, cm)
    if mode == "smoothing":
        p = fs.default_params(smoothing=1)
    else:
        p = fs.default_params(effects=3, shade=0.5, fog_start=40.0, fog_end=350.0,
                              fog_color=0xFFB0B8C8)
    specs = [(s, 0, w, h, cam) for s, (w, h) in enumerate(SIZES)
             for cam in fs.gen_walk(40 + s, hm, 2, step=2.0, yaw=0.05, above=(20, 120),
                                    distance=400.0, screen_h=h)]
    bufs = [fs.PinnedBuffer((h, w)) for (_, _, w, h, _) in specs]
    srv = fs.Server(gpu_ctx, [fmap], budget_bytes=8 << 20, nsessions=len(SIZES), max_batch=8,
                    slots=2, max_distance=400.0, params=p)
    try:
        reqs = _fill(fs, specs, bufs)
        st = srv.run(reqs)
        assert st["errors"] == 0
        for i, (s, m, w, h, cam) in enumerate(specs):
            ref = orc.render(cam, orc.params_from(p), hm, cm, w, h, threads=0)
            assert count_diff(bufs[i].array, ref) == 0, (mode, i)
    finally:
        srv.close()
        for b in bufs:
            b.close()
