"""GB300-native trajectory-similarity kNN engine.

Drop-in for the batch query path of CudaRuntime1 (DTW, LCSS, discrete
Frechet, symmetric Hausdorff, lock-step Euclidean): hand-written sm_103a CUDA
kernels behind a C ABI (include/tsim.h, libtsim.so), the reference's own
entry-point names (include/compat/), an exact kNN engine over a
device-resident database, and a continuous-batching serving loop.
"""
from . import datagen  # noqa: F401
from .api import (Context, Database, Server, execute_rtree_csr_kernel_on_gpu, knn,  # noqa: F401
                  knn_device, knn_scratch_bytes,
                  launch_dtw_batch_gpu_knn, launch_euclidean_batch_gpu_rtree_exact,
                  launch_frechet_batch_gpu_wavefront, launch_hausdorff_rtree_gpu,
                  launch_lcss_batch_gpu_wavefront_knn, make_params, ref_batch_device,
                  run_hausdorff_rtree_gpu_pipeline)
from .buildlib import build  # noqa: F401

__all__ = [
    "Context", "Database", "Server", "knn", "knn_device", "knn_scratch_bytes", "make_params",
    "ref_batch_device",
    "launch_dtw_batch_gpu_knn", "launch_lcss_batch_gpu_wavefront_knn",
    "launch_frechet_batch_gpu_wavefront", "run_hausdorff_rtree_gpu_pipeline",
    "launch_hausdorff_rtree_gpu", "launch_euclidean_batch_gpu_rtree_exact",
    "execute_rtree_csr_kernel_on_gpu", "build", "datagen",
]
