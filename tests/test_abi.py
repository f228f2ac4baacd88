"""The C-ABI library builds for sm_103a, loads, and exports every entry point
its headers declare.  No GPU is needed: nothing here launches a kernel."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def _c_api_names():
    src = open(os.path.join(ROOT, "include", "tsim.h")).read()
    return set(re.findall(r"TSIM_API\s+[\w\s\*]+?\b(tsim_\w+)\s*\(", src))


def test_every_c_entry_point_is_exported(tsim):
    names = _c_api_names()
    assert len(names) >= 19
    missing = names - _exported(tsim.build())
    assert not missing, missing


def test_reference_named_entry_points_are_exported(tsim):
    """The GPU functions of the reference's headers (dtw.cuh, lcss.cuh,
    frechet.cuh, hausdorff.cuh, euclidean.cuh) with C++ linkage and the
    reference's exact signatures."""
    syms = _exported(tsim.build())
    demangled = subprocess.run(["c++filt"], input="\n".join(sorted(syms)), capture_output=True,
                               text=True, check=True).stdout.splitlines()
    want = [
        "launch_dtw_batch_gpu_knn(Point const*, Point const*, float*, int, int, int, float&)",
        "launch_lcss_batch_gpu_wavefront_knn(Point const*, Point const*, float*, int, int, int, float, float&)",
        "launch_frechet_batch_gpu_wavefront(Point const*, Point const*, float*, int, int, int, float&)",
        "run_hausdorff_rtree_gpu_pipeline(Point const*, int, int, Point const*, int, int, float*, int)",
        "launch_hausdorff_rtree_gpu(Point const*, int, int, Point const*, int, int, int const*, int, float*, float&)",
        "launch_euclidean_batch_gpu_rtree_exact(Point const*, Point const*, float*, int, int, float&)",
        "execute_rtree_csr_kernel_on_gpu(Point const*, Point const*, int const*, int const*, float*, int, int, int, float&)",
    ]
    for w in want:
        assert w in demangled, w


def test_library_is_sm103a_only(tsim):
    lib = tsim.build()
    out = subprocess.run(["cuobjdump", "--list-elf", lib], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    arches = set(re.findall(r"sm_(\d+a?)", out.stdout))
    assert arches == {"103a"}, arches


def test_loads_and_reports_errors_without_gpu(tsim):
    import torch
    L = tsim._lib.load()
    assert L.tsim_version() >= 10000
    assert L.tsim_status_string(0) == b"ok"
    assert L.tsim_status_string(5) == b"unsupported"
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: covered by the gpu tests")
    h = C.c_void_p()
    st = L.tsim_ctx_create(0, None, C.byref(h))
    assert st != 0 and not h.value
    assert len(L.tsim_last_error()) > 0
    # null arguments are rejected before any CUDA call
    assert L.tsim_knn(None, None, None, None, 0, 0, None, None, None, None, None) == 1
    assert b"NULL" in L.tsim_last_error()


def test_python_api_raises_on_bad_input(tsim):
    with pytest.raises(ValueError):
        tsim.api._pts([[1.0, 2.0, 3.0]])
    with pytest.raises(ValueError):  # reference-named entry points check sizes first
        tsim.api.launch_dtw_batch_gpu_knn(np.zeros((10, 2), np.float32),
                                          np.zeros((10, 2), np.float32), 4, 5, 5)


C_CALLER = r"""
#include <stdio.h>
#include "tsim.h"
int main(void) {
  tsim_ctx* ctx = NULL;
  int st = tsim_ctx_create(0, NULL, &ctx);
  printf("%d %s %d\n", tsim_version(), tsim_status_string(TSIM_OK), st);
  if (st == TSIM_OK) return tsim_ctx_destroy(ctx);
  printf("%s\n", tsim_last_error());
  return 0;
}
"""

CPP_CALLER = r"""
#include <cmath>
#include <cstdio>
#include "dtw.cuh"
#include "euclidean.cuh"
#include "frechet.cuh"
#include "hausdorff.cuh"
#include "lcss.cuh"
int main() {
  Point a[8];
  for (int i = 0; i < 8; ++i) a[i] = Point{float(i), float(i % 3)};
  float out[2] = {-1.f, -1.f}, ms = 0.f;
  launch_dtw_batch_gpu_knn(a, a, out, 2, 4, 4, ms);  // each query against itself
  std::printf("%d %g %g\n", std::isnan(out[0]) ? 1 : 0, out[0], out[1]);
  return 0;
}
"""


def test_c_and_cpp_callers_build_against_the_headers(tsim, tmp_path):
    """A C caller of include/tsim.h and a C++ caller of the reference-named
    headers (include/compat/) compile, link against libtsim.so and run: the
    same steps a reference caller takes after switching libraries.  Without
    a GPU the context call fails with a status and the reference-named call
    (TSIM_COMPAT_NO_EXIT set) reports and returns NaN."""
    import shutil
    import torch
    if not (shutil.which("gcc") and shutil.which("g++")):
        pytest.skip("no host C/C++ compiler")
    libdir = os.path.dirname(tsim._lib.lib_path())
    inc = os.path.join(ROOT, "include")
    cuda_inc = "/usr/local/cuda/include"
    link = ["-L" + libdir, "-ltsim", "-Wl,-rpath," + libdir]
    (tmp_path / "c.c").write_text(C_CALLER)
    (tmp_path / "cpp.cpp").write_text(CPP_CALLER)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + inc, str(tmp_path / "c.c"),
                        "-o", str(tmp_path / "c_caller")] + link, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(inc, "compat"),
                        "-I" + cuda_inc, str(tmp_path / "cpp.cpp"), "-o", str(tmp_path / "cpp_caller")]
                       + link, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(tmp_path / "c_caller")], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    version, ok, status = out.stdout.split("\n")[0].split()
    assert int(version) >= 10000 and ok == "ok"
    assert (int(status) == 0) == torch.cuda.is_available()
    env = dict(os.environ, TSIM_COMPAT_NO_EXIT="1")
    out = subprocess.run([str(tmp_path / "cpp_caller")], capture_output=True, text=True,
                         timeout=120, env=env)
    assert out.returncode == 0, out.stderr
    nan, v0, v1 = out.stdout.split()
    if torch.cuda.is_available():
        assert nan == "0" and float(v0) == 0.0 and float(v1) == 0.0
    else:
        assert nan == "1" and "Error" in out.stderr
