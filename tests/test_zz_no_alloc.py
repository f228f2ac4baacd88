"""The allocation-free entry point tsim_ref_batch_static, called through the
C ABI, against the existing entry point tsim_ref_batch.

tsim_ref_batch_static serves callers that may not allocate device memory
(a plugin whose host application owns the GPU memory pool, a loop that cannot
afford cudaMalloc's implicit synchronisation): its scratch is a fixed array
in the library's device memory.  The two entry points run the same kernels,
so their outputs must be bit-identical -- the tolerance the other
reference-semantics tests use.  Two calls in a row check that the shared
array carries nothing over from one call to the next.  This file is collected
last; it passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu


def _static_fn(L):
    f = L.tsim_ref_batch_static
    f.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float,
                  C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_static_scratch_entry_point_matches_ref_batch(tsim):
    import torch
    from cudaruntime1_gb300 import _lib, api
    assert torch.cuda.is_available()
    L = _lib.load()
    static = _static_fn(L)
    stream = torch.cuda.Stream()
    ctx = tsim.Context(0, stream.cuda_stream)
    cases = [("dtw", 300, 96, 112, 0.5, 1), ("lcss", 200, 80, 64, 0.75, 2),
             ("frechet", 257, 70, 90, 0.5, 3)]
    with torch.cuda.stream(stream):
        for measure, num_t, n, m, eps, seed in cases:
            outs = []
            for call in range(2):  # two calls in a row on different inputs
                t1 = G.ref_base_trajectories(num_t, n, 100 * seed + call, r=300.0)
                t2 = G.ref_similar_trajectories(t1, num_t, n, m, 2.0, 200 * seed + call, r=300.0)
                d1 = torch.from_numpy(t1).cuda()
                d2 = torch.from_numpy(t2).cuda()
                want = torch.empty(num_t, dtype=torch.float32, device="cuda")
                got = torch.full((num_t,), float("nan"), dtype=torch.float32, device="cuda")
                api.ref_batch_device(ctx, measure, d1.data_ptr(), d2.data_ptr(), num_t, n, m,
                                     want.data_ptr(), eps)
                st = static(api.MEASURES[measure], d1.data_ptr(), d2.data_ptr(), num_t, n, m,
                            C.c_float(eps), got.data_ptr(), stream.cuda_stream)
                assert st == 0, L.tsim_last_error()
                stream.synchronize()
                g, w = got.cpu().numpy(), want.cpu().numpy()
                assert np.array_equal(g.view(np.uint32), w.view(np.uint32)), (measure, call)
                outs.append(g)
            assert not np.array_equal(outs[0], outs[1])
    ctx.close()


def test_static_scratch_entry_point_rejects_oversize(tsim):
    import torch
    from cudaruntime1_gb300 import _lib
    L = _lib.load()
    static = _static_fn(L)
    dummy = torch.zeros(2, dtype=torch.float32, device="cuda")
    st = static(0, dummy.data_ptr(), dummy.data_ptr(), 100000, 8, 8, C.c_float(0.5),
                dummy.data_ptr(), None)
    assert st == 5
    assert b"limit" in L.tsim_last_error()
