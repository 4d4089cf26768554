#!/usr/bin/env python3
"""Generates tests/golden/frames.json (+ frames.npz): known-answer frames of the
CPU oracle for fixed seeds, cameras and parameters; and generators.txt: digests
of the seeded input generators (height map, colour map, cameras + walk).

The reference publishes no outputs and cannot be run here, so these vectors pin
the oracle itself: across hosts (x86 here, Arm on the GPU machines) and across
changes to the repository. Each case records the bit patterns of sinf/cosf of
its yaw, so a host whose C library rounds them differently is reported as such.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import struct
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import futspace_gb300 as fs  # noqa: E402
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
_libm = C.CDLL("libm.so.6")
for _n in ("sinf", "cosf"):
    getattr(_libm, _n).restype = C.c_float
    getattr(_libm, _n).argtypes = [C.c_float]


def fbits(v: float) -> int:
    return struct.unpack("<I", struct.pack("<f", v))[0]


def maps(seed, size, rough=0.55, zero_texels=False):
    hm = fs.gen_heights(seed, size, rough)
    cm = fs.gen_colors(seed + 1, hm, 12)
    if zero_texels:
        cm = cm.copy()
        cm[::3, ::2] = 0
        cm[1::5, 1::3] = 0xFF9090E0
    return hm, cm


def cases():
    out = []
    # config 1: 320x240 over 1024^2, D=800, 40 above the local maximum; every filter pair
    hm, _ = maps(11, 1024)
    for i, cam in enumerate(fs.gen_cameras(41, hm, 3, above=(40, 40), distance=(800, 800),
                                           screen_h=240)):
        for hf in (0, 1):
            for cf in (0, 1):
                out.append(dict(map=[11, 1024, 0.55, False], cam=list(cam.as_tuple()), W=320, H=240,
                                params=[0.001, 0.0, 0.0, hf, cf, 0, 1], full=False))
    # tests/futspace.fut settings: nearest, z0=1, d=0.005, scale 240, gap = sky, 800x400
    out.append(dict(map=[11, 1024, 0.55, False],
                    cam=[512.0, 800.0, 178.0, 0.0, 100.0, 800.0, 1.0, 0xFF9090E0], W=800, H=400,
                    params=[0.005, 1.0, 240.0, 0, 0, 1, 0], full=False))
    # adversarial small frames, kept in full: zero/sky texels, integral and negative
    # coordinates, cameras below / at the terrain
    hm, _ = maps(21, 256, zero_texels=True)
    at = float(oracle.lib().fso_height_bilinear(hm.ctypes.data, 256, 256, 64.5, 64.25))
    adv = [[100.0, 100.0, 300.0, 0.0, 24.0, 200.0, 1.2, 0xFF9090E0],
           [-37.0, -300.0, 120.0, 1.5707964, 30.0, 400.0, 1.2, 0xFF9090E0],
           [64.5, 64.25, -10.0, 0.3, 24.0, 150.0, 1.2, 0xFF9090E0],
           [64.5, 64.25, at, 0.3, 24.0, 150.0, 1.2, 0xFF9090E0]]
    for cam in adv:
        for gap in (0, 1):
            out.append(dict(map=[21, 256, 0.55, True], cam=cam, W=61, H=47,
                            params=[0.001, 0.0, 0.0, 1, 1, gap, 1], full=True))
    return out


def render_case(c):
    hm, cm = maps(c["map"][0], c["map"][1], c["map"][2], c["map"][3])
    cam = dict(zip(["x", "y", "height", "angle", "horizon", "distance", "fov", "sky_color"],
                   c["cam"]))
    p = oracle.make_params(*c["params"])
    return oracle.render(cam, p, hm, cm, c["W"], c["H"], threads=0), hm, cm


def generator_digests():
    hm = fs.gen_heights(7, 256, 0.55)
    cm = fs.gen_colors(8, hm, 12)
    cams = fs.gen_cameras(9, hm, 4, above=(20, 200), distance=(400, 3000), screen_h=240)
    walk = fs.gen_walk(10, hm, 8, distance=3000.0, screen_h=1080)
    blob = b"".join(bytes(c) for c in cams + walk)
    return [hashlib.sha256(x).hexdigest() for x in (hm.tobytes(), cm.tobytes(), blob)]


def main():
    (OUT / "generators.txt").write_text("\n".join(generator_digests()) + "\n")
    meta, arrays = [], {}
    for i, c in enumerate(cases()):
        frame, _, _ = render_case(c)
        ang = np.float32(c["cam"][3])
        c = dict(c, sin_bits=fbits(_libm.sinf(ang)), cos_bits=fbits(_libm.cosf(ang)),
                 sha256=hashlib.sha256(frame.tobytes()).hexdigest())
        if c["full"]:
            arrays[f"f{i}"] = frame
        meta.append(c)
    (OUT / "frames.json").write_text(json.dumps(meta, indent=1) + "\n")
    np.savez_compressed(OUT / "frames.npz", **arrays)
    print(f"{len(meta)} cases, {len(arrays)} full frames")


if __name__ == "__main__":
    main()
