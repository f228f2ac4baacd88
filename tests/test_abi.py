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
    assert L.tsim_status_string(4) == b"bounded wait timed out"
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: covered by the gpu tests")
    h = C.c_void_p()
    st = L.tsim_ctx_create(0, None, C.byref(h))
    assert st != 0 and not h.value
    assert len(L.tsim_last_error()) > 0
    # null arguments are rejected before any CUDA call
    assert L.tsim_knn(None, None, None, None, 0, 0, None, None, None, None, None) == 1
    assert b"NULL" in L.tsim_last_error()
    # the device-side wait limit lives in device memory: without a GPU the
    # setter reports the CUDA error instead of crashing
    assert L.tsim_debug_set_wait_limit(0) != 0


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


CPP_GOLDEN_CALLER = r"""
#include <cstdio>
#include <vector>
#include "dtw.cuh"
#include "frechet.cuh"
#include "hausdorff.cuh"
#include "lcss.cuh"
// reads num_t, n, m, eps and the two AoS point sets; writes DTW, LCSS,
// Frechet and Hausdorff (R-tree pipeline, top_k 10) results, num_t each
int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int dims[3];
  float eps;
  if (std::fread(dims, sizeof(int), 3, f) != 3 || std::fread(&eps, sizeof(float), 1, f) != 1)
    return 4;
  const int num_t = dims[0], n = dims[1], m = dims[2];
  std::vector<Point> t1((size_t)num_t * n), t2((size_t)num_t * m);
  if (std::fread(t1.data(), sizeof(Point), t1.size(), f) != t1.size() ||
      std::fread(t2.data(), sizeof(Point), t2.size(), f) != t2.size())
    return 5;
  std::fclose(f);
  std::vector<float> out(4 * (size_t)num_t, -1.f);
  float ms = 0.f;
  launch_dtw_batch_gpu_knn(t1.data(), t2.data(), out.data(), num_t, n, m, ms);
  launch_lcss_batch_gpu_wavefront_knn(t1.data(), t2.data(), out.data() + num_t, num_t, n, m, eps,
                                      ms);
  launch_frechet_batch_gpu_wavefront(t1.data(), t2.data(), out.data() + 2 * num_t, num_t, n, m,
                                     ms);
  run_hausdorff_rtree_gpu_pipeline(t1.data(), num_t, n, t2.data(), num_t, m,
                                   out.data() + 3 * num_t);
  FILE* g = std::fopen(argv[2], "wb");
  if (!g || std::fwrite(out.data(), sizeof(float), out.size(), g) != out.size()) return 6;
  std::fclose(g);
  return 0;
}
"""


@pytest.mark.gpu
def test_cpp_caller_matches_reference_goldens_on_gpu(tsim, oracle, tmp_path):
    """A C++ caller written against the reference-named headers
    (include/compat/), compiled with g++ and linked against libtsim.so, runs
    on the GPU on the golden inputs: DTW, LCSS and Frechet are bit-exact
    against the reference's own CPU outputs (CudaRuntime1/dtw.cpp, lcss.cpp,
    frechet.cpp, compiled into the fixture), Hausdorff against the oracle's
    restatement of the reference's candidate loop over the same bounding-box
    candidates -- the relink path a reference user takes."""
    import shutil
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    libdir = os.path.dirname(tsim._lib.lib_path())
    inc = os.path.join(ROOT, "include")
    (tmp_path / "gold.cpp").write_text(CPP_GOLDEN_CALLER)
    exe = str(tmp_path / "gold_caller")
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(inc, "compat"),
                        "-I/usr/local/cuda/include", str(tmp_path / "gold.cpp"), "-o", exe,
                        "-L" + libdir, "-ltsim", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    z = np.load(os.path.join(ROOT, "tests", "golden", "ref_batch.npz"))
    for ci in range(int(z["ncases"][0])):
        num_t, n, m = (int(v) for v in z[f"c{ci}_meta"])
        eps = np.float32(z[f"c{ci}_eps"][0])
        t1 = np.ascontiguousarray(z[f"c{ci}_t1"], np.float32)
        t2 = np.ascontiguousarray(z[f"c{ci}_t2"], np.float32)
        inp = tmp_path / f"in{ci}.bin"
        inp.write_bytes(np.array([num_t, n, m], np.int32).tobytes() + eps.tobytes() +
                        t1.tobytes() + t2.tobytes())
        outp = tmp_path / f"out{ci}.bin"
        res = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True,
                             timeout=300)
        assert res.returncode == 0, (ci, res.stdout, res.stderr)
        got = np.fromfile(outp, np.float32).reshape(4, num_t)
        for row, meas in enumerate(("dtw", "lcss", "frechet")):
            want = z[f"c{ci}_{meas}"]
            assert np.array_equal(got[row].view(np.uint32), want.view(np.uint32)), (ci, meas)
        cand = oracle.mbr_knn(t1, n, t2, m, 10)
        want_h = oracle.ref_hausdorff_cands(t1, n, t2, m, cand)
        assert np.array_equal(got[3].view(np.uint32), want_h.view(np.uint32)), (ci, "hausdorff")


def test_product_library_has_no_bounds_checks(tsim):
    """The product library reports -1 from tsim_debug_bounds_violations: its
    shared-memory indices are unchecked (libtsim_debug.so checks them)."""
    L = tsim._lib.load()
    n, f = C.c_int64(7), C.c_int64(7)
    assert L.tsim_debug_bounds_violations(C.byref(n), C.byref(f)) == 0
    assert n.value == -1 and f.value == 0
