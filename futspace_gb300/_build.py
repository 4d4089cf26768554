"""Build recipe for the native libraries (no cmake, no setuptools).

Compiles, in parallel and in-tree:
  * futspace_gb300/_lib/libfutspace_gb300.so -- CUDA kernels for sm_103a plus
    the C host library and its C ABI (include/futspace_gb300.h, libfutspace.h);
  * oracle/_build/libfs_oracle.so -- the CPU oracle used by the tests (only
    built here because this is the one place that knows the compilers).

Floating point: nvcc gets --fmad=false and gcc -ffp-contract=off, so no
multiply-add is fused anywhere (the renderer's arithmetic must round exactly
like the reference's). No host-architecture flags: the same recipe runs on x86
and on the Arm GPU hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "futspace_gb300"
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libfutspace_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libfs_oracle.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _newer(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))


def build_library(verbose: bool = False) -> Path:
    ch = cuda_home()
    nvcc = str(ch / "bin" / "nvcc")
    inc = ["-I", str(ch / "include"), "-I", str(ROOT / "include"), "-I", str(CSRC)]
    OBJ.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJ / (src.stem + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + hdrs):
            jobs.append([nvcc, ARCH, "-O3", "--fmad=false", "-lineinfo", "-std=c++17",
                         "-Xcompiler", "-fPIC", *inc, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.c")):
        obj = OBJ / (src.stem + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + hdrs):
            jobs.append(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-ffp-contract=off",
                         "-fopenmp", "-Wall", "-Wno-unused-function", *inc, "-c", str(src),
                         "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if jobs or not _newer(LIB, objs):
        libdir = ch / "lib64"
        if not libdir.exists():
            libdir = ch / "lib"
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, ARCH, "-shared", "-cudart", "shared", "-Xcompiler", "-fopenmp", "-o",
              str(tmp), *map(str, objs), "-L", str(libdir), f"-Xlinker=-rpath={libdir}", "-lm"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    src = ORACLE_DIR / "fs_oracle.c"
    hdr = ORACLE_DIR / "fs_oracle.h"
    ORACLE_LIB.parent.mkdir(exist_ok=True)
    if not _newer(ORACLE_LIB, [src, hdr]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
              str(src), "-o", str(tmp), "-lm"])
        os.replace(tmp, ORACLE_LIB)
    if verbose:
        print(f"built {ORACLE_LIB}", file=sys.stderr)
    return ORACLE_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_library, verbose)
        b = ex.submit(build_oracle, verbose)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(verbose=True)
