// Tiled FP64 complex GEMM over one 64 x 64 output tile (a CTA of 256
// threads, 4 x 4 complex per thread, K in chunks of 16 through shared
// memory), with caller-supplied element loaders and epilogue, and the FP64
// RK4 stage kernel of the Redfield path built on it (one GEMM Y = L S per
// stage with the stage combination of lime/phys.py:636-649 in the
// epilogue).  Shared by the Redfield generator assembly, its RK4 loop and
// their adjoints.
#pragma once

#include "common.cuh"

namespace lime {
namespace rf {

constexpr int kThreads = 256;
constexpr int kTile = 64;   // CTA output tile (64 x 64), 4 x 4 complex per thread
constexpr int kKC = 16;

// Tiled complex GEMM over one output tile; loaders give A(i,k) and B(k,j)
// (zero outside), epi(i, j, value) consumes the result.
template <class LA, class LB, class EPI>
__device__ void gemm_tile(int M, int N, int K, int i0, int j0, LA la, LB lb, EPI epi) {
  __shared__ double2 As[kTile][kKC + 1];
  __shared__ double2 Bs[kKC][kTile + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double2 acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = cz();
  for (int k0 = 0; k0 < K; k0 += kKC) {
    for (int idx = threadIdx.x; idx < kTile * kKC; idx += kThreads) {
      const int r = idx / kKC, c = idx % kKC;
      const int gi = i0 + r, gk = k0 + c;
      As[r][c] = (gi < M && gk < K) ? la(gi, gk) : cz();
    }
    for (int idx = threadIdx.x; idx < kTile * kKC; idx += kThreads) {
      const int r = idx / kTile, c = idx % kTile;
      const int gk = k0 + r, gj = j0 + c;
      Bs[r][c] = (gk < K && gj < N) ? lb(gk, gj) : cz();
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kKC; ++kk) {
      double2 a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = As[ty + 16 * u][kk];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = Bs[kk][tx + 16 * v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) cfma(acc[u][v], a[u], b[v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int gi = i0 + ty + 16 * u, gj = j0 + tx + 16 * v;
      if (gi < M && gj < N) epi(gi, gj, acc[u][v]);
    }
}

// ---------------------------------------------------------------- RK4 stages
struct StageArgs {
  int D, R, stage;
  double dt;
  const double2* L;     // D x D
  const double2* S;     // stage input, D x R
  double2* P;           // state, D x R
  double2* acc;         // D x R
  double2* Snext;       // next stage input, D x R
};

static __global__ void __launch_bounds__(kThreads) stage_kernel(StageArgs a) {
  const int D = a.D, R = a.R;
  auto la = [&](int i, int k) -> double2 { return a.L[(int64_t)i * D + k]; };
  auto lb = [&](int k, int j) -> double2 { return a.S[(int64_t)k * R + j]; };
  const double dt = a.dt, dt2 = a.dt / 2.0;
  const int s = a.stage;
  auto epi = [&](int i, int j, double2 f) {
    const int64_t e = (int64_t)i * R + j;
    if (s == 0) {
      a.acc[e] = f;
      a.Snext[e] = cadd(a.P[e], cscale(f, dt2));
    } else if (s < 3) {
      a.acc[e] = cadd(a.acc[e], cscale(f, 2.0));
      a.Snext[e] = cadd(a.P[e], cscale(f, s == 2 ? dt : dt2));
    } else {
      const double2 sum = cadd(a.acc[e], f);
      const double2 nr = cadd(a.P[e], cscale(make_double2(sum.x / 6., sum.y / 6.), dt));
      a.P[e] = nr;
      a.Snext[e] = nr;
    }
  };
  gemm_tile(D, R, D, blockIdx.y * kTile, blockIdx.x * kTile, la, lb, epi);
}

}  // namespace rf
}  // namespace lime
