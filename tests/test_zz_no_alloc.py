"""The allocation-free entry point tsim_ref_batch_static, called through the
C ABI, against the existing entry point tsim_ref_batch and against the
reference's own CPU outputs.

tsim_ref_batch_static serves callers that may not allocate device memory
(a plugin whose host application owns the GPU memory pool, a loop that cannot
afford cudaMalloc's implicit synchronisation): its scratch is a fixed array
in the library's device memory.  The two entry points run the same kernels,
so their outputs must be bit-identical -- the tolerance the other
reference-semantics tests use -- and both must equal the golden outputs of
the reference's compiled CPU code bit for bit.  Two calls in a row check that
the shared array carries nothing over from one call to the next; repeated
calls must leave the device's free memory unchanged.  This file is collected
last; it passes alone in a fresh process and after the other tests.
"""
import ctypes as C
import os

import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_batch.npz")
TSIM_ERR_UNSUPPORTED = 5


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


def test_static_scratch_entry_point_matches_reference_goldens(tsim):
    """Bit-exact against the outputs of the reference's own CPU functions
    (CudaRuntime1/dtw.cpp, lcss.cpp, frechet.cpp) stored in the fixture."""
    import torch
    from cudaruntime1_gb300 import _lib, api
    L = _lib.load()
    static = _static_fn(L)
    z = np.load(GOLD)
    stream = torch.cuda.Stream()
    for ci in range(int(z["ncases"][0])):
        num_t, n, m = (int(v) for v in z[f"c{ci}_meta"])
        eps = float(z[f"c{ci}_eps"][0])
        d1 = torch.from_numpy(np.ascontiguousarray(z[f"c{ci}_t1"])).cuda()
        d2 = torch.from_numpy(np.ascontiguousarray(z[f"c{ci}_t2"])).cuda()
        for measure in ("dtw", "lcss", "frechet"):
            got = torch.full((num_t,), float("nan"), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            st = static(api.MEASURES[measure], d1.data_ptr(), d2.data_ptr(), num_t, n, m,
                        C.c_float(eps), got.data_ptr(), stream.cuda_stream)
            assert st == 0, L.tsim_last_error()
            stream.synchronize()
            want = z[f"c{ci}_{measure}"]
            assert np.array_equal(got.cpu().numpy().view(np.uint32), want.view(np.uint32)), \
                (ci, measure)


def test_static_scratch_entry_point_allocates_nothing(tsim):
    """After one warm-up call per measure (which loads the kernels), further
    calls leave the device's free memory unchanged: no arena and no
    cudaMalloc, whose 2 MiB granularity would show."""
    import torch
    from cudaruntime1_gb300 import _lib, api
    L = _lib.load()
    static = _static_fn(L)
    num_t, n, m = 500, 64, 64
    t1 = G.ref_base_trajectories(num_t, n, 7, r=300.0)
    t2 = G.ref_similar_trajectories(t1, num_t, n, m, 2.0, 8, r=300.0)
    d1 = torch.from_numpy(t1).cuda()
    d2 = torch.from_numpy(t2).cuda()
    out = torch.empty(num_t, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def calls():
        for measure in ("dtw", "lcss", "frechet"):
            st = static(api.MEASURES[measure], d1.data_ptr(), d2.data_ptr(), num_t, n, m,
                        C.c_float(0.5), out.data_ptr(), None)
            assert st == 0, L.tsim_last_error()
        torch.cuda.synchronize()

    calls()
    free0 = torch.cuda.mem_get_info()[0]
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(3):
        calls()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_reserved() == reserved0


def test_static_scratch_entry_point_size_limit(tsim):
    """The binding limit is the filter's shared memory: num_t <= 25600 - 2 m.
    At the limit the call runs and equals tsim_ref_batch; one above it is
    refused with TSIM_ERR_UNSUPPORTED, as is a far larger call."""
    import torch
    from cudaruntime1_gb300 import _lib, api
    L = _lib.load()
    static = _static_fn(L)
    n = m = 8
    lim = 25600 - 2 * m
    t1 = G.ref_base_trajectories(lim + 1, n, 31, r=300.0)
    t2 = G.ref_similar_trajectories(t1, lim + 1, n, m, 2.0, 32, r=300.0)
    d1 = torch.from_numpy(t1).cuda()
    d2 = torch.from_numpy(t2).cuda()
    got = torch.full((lim + 1,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = static(0, d1.data_ptr(), d2.data_ptr(), lim, n, m, C.c_float(0.5), got.data_ptr(), None)
    assert st == 0, L.tsim_last_error()
    torch.cuda.synchronize()
    with tsim.Context(0) as ctx:
        want = torch.empty(lim, dtype=torch.float32, device="cuda")
        api.ref_batch_device(ctx, "dtw", d1.data_ptr(), d2.data_ptr(), lim, n, m, want.data_ptr())
        ctx.synchronize()
    g = got[:lim].cpu().numpy()
    assert np.array_equal(g.view(np.uint32), want.cpu().numpy().view(np.uint32))
    assert np.isnan(got[lim].item())  # nothing written past num_t
    for num_t in (lim + 1, 100000):
        st = static(0, d1.data_ptr(), d2.data_ptr(), num_t, n, m, C.c_float(0.5),
                    got.data_ptr(), None)
        assert st == TSIM_ERR_UNSUPPORTED
        assert b"limit" in L.tsim_last_error()
