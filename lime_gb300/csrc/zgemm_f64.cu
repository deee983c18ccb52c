// Strided batched complex128 GEMM for the Liouville-space Green's-function
// route and the eigenbasis transforms of the Redfield solver
// (lime/oqs.py:169-366: U(t) = U1 exp(w t) U1^-1, expect, the 2- and 4-point
// correlation functions, and the basis changes V^dag X V of
// lime/phys.py:706-718).  Every contraction there is
//     C[z][i][j] = sum_k op(A)[z][i][k] s[z][k] op(B)[z][k][j]
// with op = identity or complex conjugate, an optional per-(z, k) complex
// scale s (the exp(w_j t_z) of the spectral propagator), and arbitrary
// element strides for rows, columns and the batch index (0 broadcasts), so
// a (D, D, Nt) propagator contracts with a block of vectors without any
// transposition.  FP64 on the tiled GEMM of gemm_f64.cuh (64 x 64 tiles).

#include "gemm_f64.cuh"

namespace lime {
namespace zg {

struct Args {
  int M, N, K;
  int conj_a, conj_b;
  const double2* A; int64_t a_rs, a_cs, a_bs;
  const double2* B; int64_t b_rs, b_cs, b_bs;
  const double2* S; int64_t s_ks, s_bs;
  double2* C; int64_t c_rs, c_cs, c_bs;
  int z0;
};

__global__ void __launch_bounds__(rf::kThreads) zgemm_kernel(Args a) {
  const int64_t z = (int64_t)a.z0 + blockIdx.z;
  const double2* A = a.A + z * a.a_bs;
  const double2* B = a.B + z * a.b_bs;
  const double2* S = a.S ? a.S + z * a.s_bs : nullptr;
  double2* C = a.C + z * a.c_bs;
  auto la = [&](int i, int k) -> double2 {
    double2 v = A[(int64_t)i * a.a_rs + (int64_t)k * a.a_cs];
    if (a.conj_a) v.y = -v.y;
    if (S != nullptr) v = cmul(v, S[(int64_t)k * a.s_ks]);
    return v;
  };
  auto lb = [&](int k, int j) -> double2 {
    double2 v = B[(int64_t)k * a.b_rs + (int64_t)j * a.b_cs];
    if (a.conj_b) v.y = -v.y;
    return v;
  };
  auto epi = [&](int i, int j, double2 v) { C[(int64_t)i * a.c_rs + (int64_t)j * a.c_cs] = v; };
  rf::gemm_tile(a.M, a.N, a.K, blockIdx.y * rf::kTile, blockIdx.x * rf::kTile, la, lb, epi);
}

}  // namespace zg
}  // namespace lime

using namespace lime;

extern "C" int lime_zgemm_strided_f64(const LimeZgemmDesc* d, void* stream) {
  if (!d || d->M <= 0 || d->N <= 0 || d->K <= 0 || d->batch <= 0) return LIME_ERR_ARG;
  if (!d->A || !d->B || !d->C) return LIME_ERR_ARG;
  if ((d->conj_a & ~1) || (d->conj_b & ~1)) return LIME_ERR_ARG;
  zg::Args a{};
  a.M = d->M; a.N = d->N; a.K = d->K;
  a.conj_a = d->conj_a; a.conj_b = d->conj_b;
  a.A = reinterpret_cast<const double2*>(d->A); a.a_rs = d->a_rs; a.a_cs = d->a_cs; a.a_bs = d->a_bs;
  a.B = reinterpret_cast<const double2*>(d->B); a.b_rs = d->b_rs; a.b_cs = d->b_cs; a.b_bs = d->b_bs;
  a.S = reinterpret_cast<const double2*>(d->scale); a.s_ks = d->s_ks; a.s_bs = d->s_bs;
  a.C = reinterpret_cast<double2*>(d->C); a.c_rs = d->c_rs; a.c_cs = d->c_cs; a.c_bs = d->c_bs;
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned gx = (unsigned)((d->N + rf::kTile - 1) / rf::kTile);
  const unsigned gy = (unsigned)((d->M + rf::kTile - 1) / rf::kTile);
  if (gy > 65535u) return LIME_ERR_UNSUPPORTED;
  int64_t launches = 0;
  for (int z0 = 0; z0 < d->batch; z0 += 65535) {
    a.z0 = z0;
    const unsigned gz = (unsigned)((d->batch - z0) < 65535 ? (d->batch - z0) : 65535);
    zg::zgemm_kernel<<<dim3(gx, gy, gz), rf::kThreads, 0, st>>>(a);
    LIME_CUDA_TRY(cudaGetLastError());
    ++launches;
  }
  count_launch(launches);
  return LIME_OK;
}
