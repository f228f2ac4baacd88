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
