// Shared device helpers for the lime_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lime_gb300.h"

namespace lime {

// adds k to the library's launch counter (lime_launch_count)
void count_launch(int64_t k = 1);

// ---------------------------------------------------------------- complex
__device__ __forceinline__ double2 cz() { return make_double2(0.0, 0.0); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// c += a * b
__device__ __forceinline__ void cfma(double2& c, double2 a, double2 b) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
}
__device__ __forceinline__ bool cfinite(double2 a) { return isfinite(a.x) && isfinite(a.y); }

// ---------------------------------------------------------------- bounds checks
// The bounds-checked build (-DLIME_CHECK, liblime_gb300_check.so) checks the
// byte range [off, off + len) of the accesses whose offsets come from tile,
// piece and instance arithmetic against the extent of their buffer: a range
// outside [0, extent) raises LIME_FLAG_BOUNDS in the kernel's status word and
// the access is skipped (never a trap).  In the regular build the check is
// compiled away.
__device__ __forceinline__ bool in_bounds(size_t off, size_t len, size_t extent, int32_t* status) {
#ifdef LIME_CHECK
  if (off > extent || len > extent - off) {
    if (status) atomicOr(status, LIME_FLAG_BOUNDS);
    return false;
  }
#else
  (void)off; (void)len; (void)extent; (void)status;
#endif
  return true;
}
constexpr size_t kNoExtent = ~(size_t)0;   // extent of a buffer the caller did not describe

// ---------------------------------------------------------------- block reductions
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = (l < NT / 32) ? red[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (l == 0) red[0] = s;
  }
  __syncthreads();
  s = red[0];
  __syncthreads();
  return s;
}

// ---------------------------------------------------------------- compensated RK4 update
// Final RK4 combination x += (acc + f) dt/6 on an fp32 pair (x, lo): dt/6 is
// the float pair c6 + c6lo, the increment's rounding error and the sum's
// two-sum error are carried in lo, so neither rounding nor the step size
// drifts over thousands of steps (lime/phys.py:636-649).
__device__ __forceinline__ float rk4_final_f32(float x, float acc, float f, float c6, float c6lo, float& lo) {
  const float ksum = __fadd_rn(acc, f);
  const float inc = __fmul_rn(ksum, c6);
  const float inc_res = __fmaf_rn(ksum, c6, -inc);
  const float inc_lo = __fmaf_rn(ksum, c6lo, inc_res);
  const float sum = __fadd_rn(x, inc);
  const float bv = __fsub_rn(sum, x);
  const float err = __fadd_rn(__fsub_rn(x, __fsub_rn(sum, bv)), __fsub_rn(inc, bv));
  float l = __fadd_rn(lo, __fadd_rn(err, inc_lo));
  const float hi2 = __fadd_rn(sum, l);
  lo = __fsub_rn(l, __fsub_rn(hi2, sum));
  return hi2;
}

}  // namespace lime

#define LIME_CUDA_TRY(expr)                            \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) return LIME_ERR_CUDA;       \
  } while (0)
