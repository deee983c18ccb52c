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
// device address; the device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on
// that device.

#include <mutex>

#include "common.cuh"

namespace {

constexpr size_t kScratchBytes = LIME_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_dev[kMaxDevices] = {nullptr};

// Device address of g_scratch on the current device (set up on first use).
int scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return LIME_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return LIME_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return LIME_ERR_CUDA;
    g_scratch_dev[dev] = p;
  }
  *out = g_scratch_dev[dev];
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
