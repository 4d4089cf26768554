"""The oracle-side generators (oracle/gen.py, numpy) against the committed
digests and against the product library's generators: the CPU reference arm
of the benchmark makes its inputs with them, without loading the product."""
import hashlib

import numpy as np
import pytest

from conftest import ROOT


def test_numpy_generators_reproduce_committed_digests():
    from oracle import gen
    golden = (ROOT / "tests" / "golden" / "generators.txt").read_text().split()
    hm = gen.heights(7, 256, 0.55)
    cm = gen.colors(8, hm, 12)
    assert hashlib.sha256(hm.tobytes()).hexdigest() == golden[0]
    assert hashlib.sha256(cm.tobytes()).hexdigest() == golden[1]
    cams = gen.cameras(9, hm, 4, above=(20, 200), distance=(400, 3000), screen_h=240)
    walk = gen.walk(10, hm, 8, distance=3000.0, screen_h=1080)
    assert hashlib.sha256(gen.camera_bytes(cams + walk)).hexdigest() == golden[2]


@pytest.mark.parametrize("seed,size,rough", [(7, 1024, 0.55), (8, 512, 0.6), (9, 2, 0.5),
                                             (10, 64, 0.9)])
def test_numpy_generators_equal_product(fs, seed, size, rough):
    from oracle import gen
    hm = gen.heights(seed, size, rough)
    np.testing.assert_array_equal(hm, fs.gen_heights(seed, size, rough))
    np.testing.assert_array_equal(gen.colors(seed + 1, hm, 12), fs.gen_colors(seed + 1, hm, 12))
    a = gen.cameras(seed + 2, hm, 5, above=(20, 200), distance=(400, 3000), screen_h=1080)
    b = fs.gen_cameras(seed + 2, hm, 5, above=(20, 200), distance=(400, 3000), screen_h=1080)
    assert gen.camera_bytes(a) == b"".join(bytes(c) for c in b)
    a = gen.walk(seed + 3, hm, 16, step=2.0, yaw=0.02, above=(30, 120), distance=3000.0,
                 screen_h=1080)
    b = fs.gen_walk(seed + 3, hm, 16, step=2.0, yaw=0.02, above=(30, 120), distance=3000.0,
                    screen_h=1080)
    assert gen.camera_bytes(a) == b"".join(bytes(c) for c in b)
