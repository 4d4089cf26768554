import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def reference_dir():
    """A checkout of the reference project (MrHootJones/futspace), named by the
    environment variable FUTSPACE_REFERENCE_DIR; None when it is not set or
    does not exist (the tests that read its files then skip)."""
    p = os.environ.get("FUTSPACE_REFERENCE_DIR")
    if not p or not Path(p).is_dir():
        return None
    return Path(p)


@pytest.fixture(scope="session", autouse=True)
def _tune_cache(tmp_path_factory):
    # keep tuning-cache writes out of the working tree
    os.environ.setdefault("FS_TUNE_CACHE", str(tmp_path_factory.mktemp("tune") / "tune.txt"))


@pytest.fixture(scope="session")
def fs():
    from futspace_gb300 import _build
    _build.build_library()
    import futspace_gb300
    futspace_gb300.lib()
    return futspace_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def maps1024(fs):
    hm = fs.gen_heights(11, 1024, 0.55)
    return hm, fs.gen_colors(12, hm, 12)


@pytest.fixture(scope="session")
def maps256(fs):
    hm = fs.gen_heights(21, 256, 0.55)
    return hm, fs.gen_colors(22, hm, 12)


@pytest.fixture(scope="session")
def gpu_ctx(fs):
    try:
        ctx = fs.Context(0)
    except fs.FsError as e:  # no device in this environment
        pytest.skip(f"no CUDA device: {e}")
    yield ctx
    ctx.close()


def count_diff(a: np.ndarray, b: np.ndarray) -> int:
    assert a.shape == b.shape, (a.shape, b.shape)
    return int(np.count_nonzero(a != b))
