// FP64 Lindblad RK4 without any device allocation by the caller.
//
// Some callers cannot hand this library a scratch buffer: a host framework
// whose memory pool owns the whole GPU and forbids foreign cudaMalloc, a
// latency-critical loop in which cudaMalloc/cudaFree would implicitly
// synchronise the device, or an application that must keep a fixed device
// footprint after start-up.  For them, lime_lindblad_rk4_f64_noalloc runs the
// same FP64 propagator as lime_lindblad_rk4_f64 with its workspace taken from
// a fixed array that lives in this library's own device image.
//
// The array is a file-scope __device__ variable, so every GPU on which the
// library is loaded holds LIME_NOALLOC_SCRATCH_BYTES of it until the process
// exits.  In host code its name only denotes a host-side stand-in, never a
// device address; the device address is looked up with cudaGetSymbolAddress,
// with the device current, on the first call in each CUDA context: the cache
// is keyed on the context's process-unique ID (cuCtxGetId), so a new context
// on the same device (after cudaDeviceReset, or a context the caller made
// current) looks the address up again instead of reusing a stale one.

#include <cuda.h>

#include <mutex>

#include "common.cuh"

namespace {

constexpr size_t kScratchBytes = LIME_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct Entry {
  unsigned long long ctx_id;   // context the address belongs to (0: none cached)
  void* ptr;
};

std::mutex g_mu;
Entry g_scratch_dev[kMaxDevices] = {};

// ID of the current context, or 0 when none is current.  The two driver
// calls are fetched through the runtime (cudaGetDriverEntryPointByVersion),
// so the library needs the driver library only once a GPU is used.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return 0;
    get_current = reinterpret_cast<GetCurrent>(f1);
    get_id = reinterpret_cast<GetId>(f2);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_scratch in the current context (looked up on the first
// call in each context).
int scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return LIME_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return LIME_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  unsigned long long id = current_context_id();
  Entry& e = g_scratch_dev[dev];
  if (id != 0 && e.ptr && e.ctx_id == id) {
    *out = e.ptr;
    return LIME_OK;
  }
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return LIME_ERR_CUDA;
  if (id == 0) id = current_context_id();   // the lookup made the device's context current
  e.ctx_id = id;
  e.ptr = id != 0 ? p : nullptr;            // no ID: look it up again next time
  *out = p;
  return LIME_OK;
}

}  // namespace

extern "C" size_t lime_noalloc_scratch_bytes(void) { return kScratchBytes; }

extern "C" int lime_lindblad_rk4_f64_noalloc(const LimeLindbladDesc* d, void* stream) {
  if (!d) return LIME_ERR_ARG;
  if (d->n <= 0 || d->batch <= 0 || d->k_dense < 0) return LIME_ERR_ARG;
  const size_t need = lime_lindblad_rk4_f64_workspace(d->n, d->batch, d->k_dense);
  if (need == 0) return LIME_ERR_ARG;
  if (need > kScratchBytes) return LIME_ERR_SCRATCH_LIMIT;
  void* scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != LIME_OK) return rc;
  // Every workspace word the propagator reads is written earlier in the same
  // call (stage buffers from rho, accumulators at stage 0, the start trace at
  // step 0), so the previous call's contents need no clearing.
  LimeLindbladDesc local = *d;
  local.workspace = scratch;
  local.workspace_bytes = kScratchBytes;
  return lime_lindblad_rk4_f64(&local, stream);
}
