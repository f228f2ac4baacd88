"""In-tree build of libtsim.so (nvcc, sm_103a only, no CMake).

Each ``csrc/*.cu`` is compiled to an object in parallel, then linked into
``cudaruntime1_gb300/libtsim.so``.  Rebuilds only when a source or header is
newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtsim.so")
# the bounds-checked build (TSIM_DEBUG_BOUNDS): tests only, built on demand
DEBUG_BUILD = os.path.join(PKG, "_build_debug")
DEBUG_LIB = os.path.join(PKG, "libtsim_debug.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def common_flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
                   "-I" + os.path.join(ROOT, "include")]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "compat", "*.cuh"))


def up_to_date(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(src: str, extra, build_dir: str = BUILD) -> str:
    obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + common_flags() + list(extra) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra=(), debug_bounds: bool = False) -> str:
    """Build libtsim.so, or with ``debug_bounds`` libtsim_debug.so (every
    shared-memory index of the DP and pairwise kernels checked)."""
    lib, bdir = (DEBUG_LIB, DEBUG_BUILD) if debug_bounds else (LIB, BUILD)
    extra = tuple(extra) + (("-DTSIM_DEBUG_BOUNDS",) if debug_bounds else ())
    if not force and up_to_date(lib):
        return lib
    os.makedirs(bdir, exist_ok=True)
    srcs = _sources()
    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, bdir), srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
