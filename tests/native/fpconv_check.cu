// Host build of the FP64-free conversions (lime_gb300/csrc/fpconv.cuh)
// checked bit for bit against the host's own conversion instructions, which
// round to nearest even like the GPU's.  Prints "ok <count>" or the first
// mismatch.  Built and run by tests/test_fpconv_host.py.
#include <stdio.h>
#include <stdint.h>
#include <string.h>
#include <cmath>
#include <random>

#include "fpconv.cuh"

using namespace lime::fpconv;

static int check_split(double v) {
  float hi, lo;
  split_f64(v, hi, lo);
  const float rh = (float)v;
  const float rl = (float)(v - (double)rh);
  if (std::isnan(v)) return std::isnan(hi) ? 0 : 1;
  if (bits32(hi) != bits32(rh) || (bits32(lo) != bits32(rl) && !(std::isnan(lo) && std::isnan(rl)))) {
    printf("split mismatch v=%.17g (%016llx): hi %08x vs %08x, lo %08x vs %08x\n", v,
           (unsigned long long)bits64(v), bits32(hi), bits32(rh), bits32(lo), bits32(rl));
    return 1;
  }
  return 0;
}

static int check_widen(float x) {
  if (std::isnan(x)) return std::isnan(widen_f32(x)) ? 0 : 1;
  if (bits64(widen_f32(x)) != bits64((double)x)) {
    printf("widen mismatch %08x\n", bits32(x));
    return 1;
  }
  return 0;
}

static int check_scale(double d, int e) {
  const double a = scale_pow2(d, e), b = std::ldexp(d, e);
  if (std::isnan(d)) return std::isnan(a) ? 0 : 1;
  if (bits64(a) != bits64(b)) {
    printf("scale mismatch d=%.17g e=%d\n", d, e);
    return 1;
  }
  return 0;
}

int main() {
  std::mt19937_64 g(20261204);
  long count = 0;
  int bad = 0;
  // random bit patterns over every exponent, and values near the edges of the fast path
  for (int i = 0; i < 2000000 && !bad; ++i, ++count) {
    uint64_t u = g();
    if (i % 4 == 1) {   // exponents near the fast-path bounds and around 1
      static const int edges[] = {896, 897, 898, 947, 948, 949, 950, 1022, 1023, 1024, 1148, 1149, 1150, 1151};
      const uint64_t E = (uint64_t)edges[g() % 14];
      u = (u & 0x800FFFFFFFFFFFFFull) | (E << 52);
    } else if (i % 4 == 2) {   // rounding ties and near-ties of the 24-bit hi
      const uint64_t E = 900 + g() % 250;
      uint64_t m = g() & 0xFFFFFE0000000ull;
      const uint64_t r = 0x10000000ull + (uint64_t)((int64_t)(g() % 3) - 1);
      m |= r & 0x1FFFFFFFull;
      u = (u & 0x8000000000000000ull) | (E << 52) | m;
    } else if (i % 4 == 3) {   // mantissas that carry into the next exponent
      const uint64_t E = 900 + g() % 250;
      u = (u & 0x8000000000000000ull) | (E << 52) | (0xFFFFFFFFFFFFFull - (g() % 0x40000000ull));
    }
    const double v = from_bits64(u);
    bad |= check_split(v);
    bad |= check_scale(v, (int)(g() % 121) - 60);
    bad |= check_widen(from_bits32((uint32_t)g()));
  }
  const double special[] = {0.0, -0.0, 1.0, -1.0, 1e-300, -1e-310, 4.9e-324, 1e300, INFINITY, -INFINITY,
                            NAN, 3.4028234663852886e38, 3.4028235677973366e38, 1.1754943508222875e-38,
                            5.2939559203393771e-23, 0.1, 1.0 / 3.0};
  for (double v : special) {
    bad |= check_split(v);
    bad |= check_scale(v, 7);
    bad |= check_scale(v, -7);
    bad |= check_widen((float)v);
    ++count;
  }
  const float fspecial[] = {1e-45f, -1e-45f, 1.1754942e-38f, 3.4028235e38f, -0.0f, 0.0f, INFINITY};
  for (float x : fspecial) bad |= check_widen(x);
  if (bad) return 1;
  printf("ok %ld\n", count);
  return 0;
}
