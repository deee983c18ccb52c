// Library-level C ABI: device check, status strings, version.
#include <atomic>

#include "common.cuh"

extern "C" int lime_device_check(void) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return LIME_ERR_NO_DEVICE;
  int major = 0, minor = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return LIME_ERR_CUDA;
  if (cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) return LIME_ERR_CUDA;
  return (major == 10 && minor == 3) ? LIME_OK : LIME_ERR_NO_DEVICE;
}

extern "C" const char* lime_status_string(int status) {
  switch (status) {
    case LIME_OK: return "ok";
    case LIME_ERR_ARG: return "invalid argument (size, stride, pointer or alignment)";
    case LIME_ERR_UNSUPPORTED: return "request not supported by this build";
    case LIME_ERR_CUDA: return "CUDA runtime error";
    case LIME_ERR_NO_DEVICE: return "no compute capability 10.3 device is current";
    case LIME_ERR_WORKSPACE: return "workspace too small";
    case LIME_ERR_SCRATCH_LIMIT:
      return "request needs more workspace than the no-allocation entry point's fixed scratch";
    default: return "unknown status";
  }
}

extern "C" int lime_version(void) { return 100; }

namespace lime {
static std::atomic<int64_t> g_launches{0};
void count_launch(int64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
}  // namespace lime

extern "C" int64_t lime_launch_count(void) { return lime::g_launches.load(std::memory_order_relaxed); }
