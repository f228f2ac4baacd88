// ref_static.cu -- the reference-semantics batch call without any device
// allocation: its scratch lives in a fixed-size array in the library's own
// device memory instead of a context arena.
//
// Who needs it: code that must not call cudaMalloc -- for instance a plugin
// running inside a host application that owns every byte of device memory
// through its own pool, or a latency-critical loop that cannot afford the
// implicit device synchronisation cudaMalloc/cudaFree may cause.  Such a
// caller passes its own inputs, outputs and stream; nothing else is needed.
//
// Costs and limits:
//  - every GPU that loads libtsim.so holds TSIM_STATIC_SCRATCH_BYTES of
//    device memory for the array until the process exits;
//  - the binding limit is shared memory, not the array: the envelope filter
//    keeps the candidate keys (8 num_t bytes) and the envelopes (16 m bytes)
//    in 200 KiB, so num_t <= 25,600 - 2 m; the array (about 136 num_t bytes)
//    would allow some 30,800 queries;
//  - all calls share the one array per device: calls that overlap on the GPU
//    (concurrent streams, or host threads) race and must be serialised by
//    the caller;
//  - the array keeps the previous call's contents; every scratch entry this
//    path reads is written earlier in the same call, so nothing is cleared.
#include <cuda.h>  // CUcontext and CUresult only: the driver is reached through the runtime

#include <mutex>

#include "tsim_internal.cuh"

namespace {

// Scratch of tsim_ref_batch_static, one copy per device that loads the library.
static __device__ __align__(256) unsigned char g_ref_static_scratch[TSIM_STATIC_SCRATCH_BYTES];

// In host code `g_ref_static_scratch` names a host-side stand-in, not device
// memory: a kernel given that name would fault (or, where the GPU can reach
// host memory, silently use the wrong memory).  Its device address is looked
// up with cudaGetSymbolAddress in the CUDA context current at the call, and
// that address is valid in that context only: the runtime's primary context
// of a device, a driver-API context the caller made current, or the primary
// context created again after cudaDeviceReset each load the module anew.  The
// addresses are therefore cached per context, keyed by the context's unique
// id (cuCtxGetId: ids are never reused within a process), so a lookup happens
// once per device and context.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

constexpr int kCacheSlots = 64;
struct Slot {
  unsigned long long ctx_id;
  void* addr;
};
std::mutex g_mu;
Slot g_cache[kCacheSlots];
int g_used = 0, g_next = 0;  // filled slots; the slot the next insertion replaces when full
CtxGetCurrentFn g_get_current = nullptr;
CtxGetIdFn g_get_id = nullptr;

int resolve_driver_calls() {
  if (g_get_current && g_get_id) return TSIM_OK;
  cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
  cudaError_t e = cudaGetDriverEntryPointByVersion(
      "cuCtxGetCurrent", reinterpret_cast<void**>(&g_get_current), 12000, cudaEnableDefault, &q1);
  if (e == cudaSuccess)
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", reinterpret_cast<void**>(&g_get_id), 12000,
                                         cudaEnableDefault, &q2);
  if (e != cudaSuccess)
    return tsim::cuda_fail(e, "cudaGetDriverEntryPointByVersion", __FILE__, __LINE__);
  if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !g_get_current ||
      !g_get_id) {
    g_get_current = nullptr;
    g_get_id = nullptr;
    return tsim::fail(TSIM_ERR_UNSUPPORTED,
                      "tsim_ref_batch_static: the driver lacks cuCtxGetCurrent/cuCtxGetId");
  }
  return TSIM_OK;
}

// id of the context current on this thread (0 and ok when none is current)
int current_context_id(unsigned long long* id) {
  CUcontext c = nullptr;
  *id = 0;
  if (g_get_current(&c) != CUDA_SUCCESS)
    return tsim::fail(TSIM_ERR_CUDA, "tsim_ref_batch_static: cuCtxGetCurrent failed");
  if (c && g_get_id(c, id) != CUDA_SUCCESS)
    return tsim::fail(TSIM_ERR_CUDA, "tsim_ref_batch_static: cuCtxGetId failed");
  return TSIM_OK;
}

int scratch_address(char** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  TSIM_TRY(resolve_driver_calls());
  unsigned long long id = 0;
  TSIM_TRY(current_context_id(&id));
  if (id != 0)
    for (int s = 0; s < g_used; ++s)
      if (g_cache[s].ctx_id == id) {
        *out = static_cast<char*>(g_cache[s].addr);
        return TSIM_OK;
      }
  // first call in this context (or no context current yet: the lookup makes
  // the runtime's context for the current device current)
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_ref_static_scratch);
  if (e != cudaSuccess) return tsim::cuda_fail(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
  if (id == 0) TSIM_TRY(current_context_id(&id));
  if (id != 0) {
    const int s = g_used < kCacheSlots ? g_used++ : (g_next++ % kCacheSlots);
    g_cache[s] = Slot{id, p};
  }
  *out = static_cast<char*>(p);
  return TSIM_OK;
}

}  // namespace

extern "C" int tsim_ref_batch_static(int measure, const tsim_point* d_t1, const tsim_point* d_t2,
                                     int num_t, int n, int m, float epsilon, float* d_out,
                                     void* stream) {
  TSIM_CHECK_ARG(measure == TSIM_DTW || measure == TSIM_LCSS || measure == TSIM_FRECHET,
                 "measure must be DTW, LCSS or Frechet");
  TSIM_CHECK_ARG(num_t >= 1 && n >= 1 && m >= 1, "num_t, n and m must be >= 1");
  TSIM_CHECK_ARG(d_t1 && d_t2 && d_out, "NULL device pointer");
  bool keys_in_smem = false;
  const size_t need = tsim::ref_scratch_bytes(num_t, m, &keys_in_smem);
  if (!keys_in_smem || need > TSIM_STATIC_SCRATCH_BYTES)
    return tsim::fail(TSIM_ERR_UNSUPPORTED,
                      "tsim_ref_batch_static: num_t=" + std::to_string(num_t) + ", m=" +
                          std::to_string(m) + " exceeds the limit (num_t <= 25600 - 2 m for the "
                          "filter's 200 KiB of shared memory; " + std::to_string(need) +
                          " bytes of a " + std::to_string(TSIM_STATIC_SCRATCH_BYTES) +
                          "-byte scratch array); use tsim_ref_batch");
  int device = 0;
  TSIM_CUDA(cudaGetDevice(&device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (st) {  // the kernels run on the current device: the stream must be one of its own
    int sdev = -1;
    TSIM_CUDA(cudaStreamGetDevice(st, &sdev));
    TSIM_CHECK_ARG(sdev == device, "the stream belongs to another device than the current one");
  }
  char* scratch = nullptr;
  TSIM_TRY(scratch_address(&scratch));
  // a context on the stack: device, stream and SM count only, no allocation
  tsim_ctx ctx;
  ctx.device = device;
  ctx.stream = st;
  TSIM_CUDA(cudaDeviceGetAttribute(&ctx.num_sms, cudaDevAttrMultiProcessorCount, device));
  return tsim::ref_batch_core(&ctx, measure, reinterpret_cast<const float2*>(d_t1),
                              reinterpret_cast<const float2*>(d_t2), num_t, n, m, epsilon, d_out,
                              scratch);
}
