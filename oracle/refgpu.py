"""The reference's own GPU kernels as a comparison column (test and bench
infrastructure only; never part of the product).

``make -C oracle refgpu REF=<dir>`` compiles the device code of the
reference's CudaRuntime1/{dtw,lcss,frechet,hausdorff,euclidean}.cu for sm_103a
into oracle/_ref/ref_<measure>.cubin, straight from the reference sources.
This module loads those cubins through the CUDA driver API (ctypes on
libcuda, in the context current on the calling thread -- torch's) and
launches the kernels with the launch shapes the reference's host code uses:

* lb_keogh_filter_kernel / lcss_strict_bound_filter_kernel /
  frechet_lb_filter_kernel: 16 x 16 blocks over the num_t x num_t matrix
  (CudaRuntime1/dtw.cu:147-149, lcss.cu:162-164, frechet.cu:167-169);
* dtw_refine_kernel: one block of min(256, (min(n,m)/32+1)*32) threads per
  pair, 3 (n+1) floats of shared memory (dtw.cu:185-192);
* lcss_refine_kernel_m_1: 256 threads, 3 n ints (lcss.cu:205-210);
* frechet_refine_kernel_m: min(min(n,m), 256) threads, 3 n floats
  (frechet.cu:205-212);
* hausdorff_tiled_rtree_kernel: one block of 256 per query (hausdorff.cu:161);
* euclidean_rtree_csr_kernel_global: one block of 256 per query
  (euclidean.cu:100).

The host steps between them (envelopes, top-10 selection, final reduce) are
restated here in numpy as the reference's host code does them
(dtw.cu:107-122, 161-176, 204-219 and the LCSS / Frechet twins).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
KERNELS = {
    "dtw": ("lb_keogh_filter_kernel", "dtw_refine_kernel"),
    "lcss": ("lcss_strict_bound_filter_kernel", "lcss_refine_kernel_m_1"),
    "frechet": ("frechet_lb_filter_kernel", "frechet_refine_kernel_m"),
    "hausdorff": ("hausdorff_tiled_rtree_kernel",),
    "euclidean": ("euclidean_rtree_csr_kernel_global",),
}
CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8


def cubin_path(measure: str) -> str:
    return os.path.join(REF_DIR, f"ref_{measure}.cubin")


def available() -> str | None:
    """None when every cubin is present, else the reason they are not."""
    missing = [m for m in KERNELS if not os.path.exists(cubin_path(m))]
    if missing:
        return ("reference kernels not built (oracle/_ref/ref_*.cubin are compiled from the "
                "reference sources by `make -C oracle refgpu`, where the reference checkout is): "
                "missing " + ",".join(missing))
    return None


class Driver:
    """The few driver-API calls the comparison needs."""

    def __init__(self):
        self.L = C.CDLL("libcuda.so.1")
        vp = C.c_void_p
        self.L.cuModuleLoad.argtypes = [C.POINTER(vp), C.c_char_p]
        self.L.cuModuleGetFunctionCount.argtypes = [C.POINTER(C.c_uint), vp]
        self.L.cuModuleEnumerateFunctions.argtypes = [C.POINTER(vp), C.c_uint, vp]
        self.L.cuFuncGetName.argtypes = [C.POINTER(C.c_char_p), vp]
        self.L.cuFuncSetAttribute.argtypes = [vp, C.c_int, C.c_int]
        self.L.cuLaunchKernel.argtypes = [vp, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                          C.c_uint, C.c_uint, vp, C.POINTER(vp), C.POINTER(vp)]
        self.L.cuModuleUnload.argtypes = [vp]

    def check(self, r, what):
        if r != 0:
            raise RuntimeError(f"{what} failed: CUresult {r}")

    def load(self, path):
        """Module handle and {unmangled kernel name: function handle}."""
        mod = C.c_void_p()
        self.check(self.L.cuModuleLoad(C.byref(mod), path.encode()), "cuModuleLoad " + path)
        cnt = C.c_uint()
        self.check(self.L.cuModuleGetFunctionCount(C.byref(cnt), mod), "cuModuleGetFunctionCount")
        fns = (C.c_void_p * cnt.value)()
        self.check(self.L.cuModuleEnumerateFunctions(fns, cnt.value, mod),
                   "cuModuleEnumerateFunctions")
        out = {}
        for f in fns:
            nm = C.c_char_p()
            self.check(self.L.cuFuncGetName(C.byref(nm), f), "cuFuncGetName")
            mangled = nm.value.decode()
            for want in sum(KERNELS.values(), ()):
                if want in mangled:  # Itanium mangling: _Z<len><name>...
                    out[want] = f
        return mod, out

    def launch(self, f, grid, block, smem, stream, args):
        """args: list of ctypes values, passed by address."""
        if smem > 48 * 1024:
            self.check(self.L.cuFuncSetAttribute(
                f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, smem), "cuFuncSetAttribute")
        params = (C.c_void_p * len(args))(*[C.cast(C.byref(a), C.c_void_p) for a in args])
        g = tuple(grid) + (1,) * (3 - len(grid))
        b = tuple(block) + (1,) * (3 - len(block))
        self.check(self.L.cuLaunchKernel(f, g[0], g[1], g[2], b[0], b[1], b[2], smem,
                                         C.c_void_p(stream), params, None), "cuLaunchKernel")


def envelopes(t, num_t, n, r=5):
    """The r = 5 sliding bounding boxes of each query point, float32
    {min_x, max_x, min_y, max_y} (CudaRuntime1/dtw.cu:107-122)."""
    p = np.asarray(t, np.float32).reshape(num_t, n, 2)
    env = np.empty((num_t, n, 4), np.float32)
    for i in range(n):
        s, e = max(0, i - r), min(n - 1, i + r)
        w = p[:, s:e + 1]
        env[:, i, 0] = w[..., 0].min(1)
        env[:, i, 1] = w[..., 0].max(1)
        env[:, i, 2] = w[..., 1].min(1)
        env[:, i, 3] = w[..., 1].max(1)
    return env.reshape(-1, 4)


def top_pairs(mat, num_t, K, descending):
    """The K best candidates per query by (bound, index) -- (bound desc,
    index) for LCSS -- as int2 pairs (dtw.cu:161-176, lcss.cpp:67-70)."""
    mat = np.asarray(mat, np.float32).reshape(num_t, num_t)
    idx = np.arange(num_t)
    out = np.empty((num_t, K, 2), np.int32)
    for q in range(num_t):
        key = -mat[q] if descending else mat[q]
        order = np.lexsort((idx, key))[:K]
        out[q, :, 0] = q
        out[q, :, 1] = order
    return out.reshape(-1, 2)
