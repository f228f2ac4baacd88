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
//  - all calls share the one array per device: calls that overlap on the GPU
//    (concurrent streams, or host threads) race and must be serialised by
//    the caller;
//  - the array keeps the previous call's contents; every scratch entry this
//    path reads is written earlier in the same call, so nothing is cleared.
#include <mutex>

#include "tsim_internal.cuh"

namespace {

// Scratch of tsim_ref_batch_static, one copy per device that loads the library.
static __device__ __align__(256) unsigned char g_ref_static_scratch[TSIM_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// In host code `g_ref_static_scratch` names a host-side stand-in, not device
// memory: a kernel given that name would fault (or, where the GPU can reach
// host memory, silently use the wrong memory).  The device address is looked
// up once per device, with that device current, and cached.
int scratch_address(int device, char** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (device < 0 || device >= kMaxDevices)
    return tsim::fail(TSIM_ERR_UNSUPPORTED, "tsim_ref_batch_static: device index out of range");
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_ref_static_scratch);
    if (e != cudaSuccess) return tsim::cuda_fail(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
    g_scratch_addr[device] = p;
  }
  *out = static_cast<char*>(g_scratch_addr[device]);
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
                          std::to_string(m) + " needs " + std::to_string(need) +
                          " bytes of scratch (limit " + std::to_string(TSIM_STATIC_SCRATCH_BYTES) +
                          ") or more shared memory than the filter has; use tsim_ref_batch");
  int device = 0;
  TSIM_CUDA(cudaGetDevice(&device));
  char* scratch = nullptr;
  TSIM_TRY(scratch_address(device, &scratch));
  // a context on the stack: device, stream and SM count only, no allocation
  tsim_ctx ctx;
  ctx.device = device;
  ctx.stream = static_cast<cudaStream_t>(stream);
  TSIM_CUDA(cudaDeviceGetAttribute(&ctx.num_sms, cudaDevAttrMultiProcessorCount, device));
  return tsim::ref_batch_core(&ctx, measure, reinterpret_cast<const float2*>(d_t1),
                              reinterpret_cast<const float2*>(d_t2), num_t, n, m, epsilon, d_out,
                              scratch);
}
