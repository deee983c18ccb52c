// Conversions between FP64 and fp32 pairs without the FP64 pipe.
//
// FP64 arithmetic and the FP64 <-> FP32 conversion instructions run at a few
// operations per clock per SM on this part, so a kernel that loads or stores
// FP64 data in bulk (the split-precision kernels' initial states, final
// states and observables) spends most of its fixed cost on them.  These
// helpers do the same conversions with integer and fp32 instructions and
// give bit-identical results to the conversion instructions:
//
//   split_f64(v, hi, lo)  hi = (float) v, lo = (float)(v - (double) hi)
//                         (round to nearest even), for |v| in
//                         [2^-74, 2^127); zeros exactly; every other value
//                         (tiny, huge, inf, nan) through the FP64
//                         instructions
//   widen_f32(x)          (double) x, exact; subnormal inputs through the
//                         conversion instruction
//   scale_pow2(d, e)      d * 2^e for a double whose result stays normal
//                         (exponent-field add), else d * 2^e in FP64
//
// They are __host__ __device__ so that a host build can check them against
// the host's own conversions bit for bit.
#pragma once

#include <stdint.h>
#include <string.h>

#include <cmath>

namespace lime {
namespace fpconv {

__host__ __device__ __forceinline__ uint64_t bits64(double v) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t u;
  memcpy(&u, &v, 8);
  return u;
#endif
}
__host__ __device__ __forceinline__ double from_bits64(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double v;
  memcpy(&v, &u, 8);
  return v;
#endif
}
__host__ __device__ __forceinline__ uint32_t bits32(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}
__host__ __device__ __forceinline__ float from_bits32(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

// v = hi + lo as two floats.  Fast path: the biased exponent E of v in
// [949, 1149], i.e. 2^-74 <= |v| < 2^127, so that hi is a normal float and
// the residual scale 2^(E - 1075) is a normal float too.  The 53-bit
// significand M is rounded to 24 bits (nearest even) for hi; the residual
// d = M - (rounded M), |d| <= 2^28, is an exact integer whose float
// rounding (I2F, nearest even) scaled by the power of two equals the float
// rounding of v - hi.
__host__ __device__ __forceinline__ void split_f64(double v, float& hi, float& lo) {
  const uint64_t u = bits64(v);
  const int E = (int)((u >> 52) & 0x7FF);
  const uint32_t sgn = (uint32_t)(u >> 63) << 31;
  if ((u << 1) == 0) {   // +-0 (v - hi is +0 either way)
    hi = from_bits32(sgn);
    lo = 0.f;
    return;
  }
  if (E < 949 || E > 1149) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
    return;
  }
  const uint64_t M = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  uint32_t q = (uint32_t)(M >> 29);                  // 24 bits, [2^23, 2^24)
  const uint32_t r = (uint32_t)(M & 0x1FFFFFFFu);     // 29 bits
  const bool up = r > 0x10000000u || (r == 0x10000000u && (q & 1u));
  const int32_t d = up ? (int32_t)r - 0x20000000 : (int32_t)r;
  q += up ? 1u : 0u;
  int eb = E - 1023 + 127;
  if (q == (1u << 24)) {   // rounded up to the next power of two
    q >>= 1;
    ++eb;
  }
  hi = from_bits32(sgn | ((uint32_t)eb << 23) | (q & 0x7FFFFFu));
  // 2^(E - 1075) as a float: biased exponent E - 1075 + 127 = E - 948 in [1, 201]
  const float scale = from_bits32((uint32_t)(E - 948) << 23);
  const float l = (float)d * scale;                  // exact: a power-of-two scaling of a normal result
  lo = (sgn && d != 0) ? -l : l;   // an exact residual is +0, as v - hi gives
}

// (double) x, exact.
__host__ __device__ __forceinline__ double widen_f32(float x) {
  const uint32_t u = bits32(x);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint64_t s = (uint64_t)(u >> 31) << 63;
  if (e == 0) {
    if ((u & 0x7FFFFFu) == 0) return from_bits64(s);
    return (double)x;   // subnormal
  }
  const uint64_t ed = (e == 0xFFu) ? 0x7FFull : (uint64_t)(e - 127 + 1023);
  return from_bits64(s | (ed << 52) | ((uint64_t)(u & 0x7FFFFFu) << 29));
}

// d * 2^e (exact).  Exponent-field add when d and the result are normal.
__host__ __device__ __forceinline__ double scale_pow2(double d, int e) {
  const uint64_t u = bits64(d);
  const int E = (int)((u >> 52) & 0x7FF);
  if (E == 0 || E == 0x7FF || E + e < 1 || E + e > 0x7FE) {
#ifdef __CUDA_ARCH__
    return d * __longlong_as_double((long long)((uint64_t)(1023 + e) << 52));
#else
    return std::ldexp(d, e);
#endif
  }
  return from_bits64(u + ((uint64_t)(int64_t)e << 52));
}

}  // namespace fpconv
}  // namespace lime
