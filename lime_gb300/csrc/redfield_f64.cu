// Bloch-Redfield generator assembly and FP64 RK4 on vec(rho) (sm_103a).
//
// Generator (lime/oqs.py:528-579), in the eigenbasis of H with row-major
// Liouville index (a, b) -> a N + b (lime/superoperator.py:131-151):
//   L[ab, cd] = -i (E_a - E_b) d_ac d_bd - d_bd P_ac - d_ac Q_db
//               + sum_k ( A_k[a,c] conj(Lam_k[b,d]) + Lam_k[a,c] A_k[d,b] )
// with Lam_k = C_k o A_k, P = sum_k A_k Lam_k, Q = sum_k Lam_k^dag A_k.  This
// is the closed form of -1j op2sop(diag E) - sum_k op2sop(A_k)(left(Lam_k) -
// right(Lam_k^dag)); the O(N^4 K) sum is one GEMM U (N^2 x 2K) . V (2K x N^2)
// whose epilogue scatters (a,c),(d,b) to (ab, cd) and adds the local terms.
//
// Time stepping (lime/oqs.py:373-472): RK4 on the right-hand-side block
// P (D x R, column r = vec rho_r) with one GEMM Y = L S per stage and the
// stage combination fused into the GEMM epilogue.  FP64 throughout; this is
// the exact path (DFMA-bound on GB300).

#include "gemm_f64.cuh"

namespace lime {
namespace rf {

// ---------------------------------------------------------------- assembly
__global__ void lam_kernel(int n, int k, const double2* A, const double* C, int64_t c_stride, double2* Lam) {
  const int64_t nn = (int64_t)n * n;
  const int64_t total = (int64_t)k * nn;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    Lam[e] = cscale(A[e], C[(e / nn) * c_stride + e % nn]);
}

// P = sum_k A_k Lam_k, Q = sum_k Lam_k^dag A_k (one element per thread)
__global__ void pq_kernel(int n, int k, const double2* A, const double2* Lam, double2* P, double2* Q) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    double2 p = cz(), q = cz();
    for (int kk = 0; kk < k; ++kk) {
      const double2* Ak = A + kk * nn;
      const double2* Lk = Lam + kk * nn;
      for (int m = 0; m < n; ++m) {
        cfma(p, Ak[(int64_t)i * n + m], Lk[(int64_t)m * n + j]);
        cfma(q, cconj(Lk[(int64_t)m * n + i]), Ak[(int64_t)m * n + j]);
      }
    }
    P[e] = p;
    Q[e] = q;
  }
}

struct BuildArgs {
  int n, k;
  const double* E;
  const double2* A;
  const double2* Lam;
  const double2* P;
  const double2* Q;
  double2* R;
};

__global__ void __launch_bounds__(kThreads) assemble_kernel(BuildArgs a) {
  const int n = a.n, K = a.k;
  const int64_t nn = (int64_t)n * n;
  const int D = n * n;
  // U[(a,c), kk] = kk < K ? A_kk[a,c] : Lam_{kk-K}[a,c]
  auto la = [&](int row, int kk) -> double2 {
    return kk < K ? a.A[kk * nn + row] : a.Lam[(kk - K) * nn + row];
  };
  // V[kk, (d,b)] = kk < K ? conj(Lam_kk[b,d]) : A_{kk-K}[d,b]
  auto lb = [&](int kk, int col) -> double2 {
    const int d = col / n, b = col % n;
    return kk < K ? cconj(a.Lam[kk * nn + (int64_t)b * n + d]) : a.A[(kk - K) * nn + col];
  };
  auto epi = [&](int row, int col, double2 v) {
    const int ai = row / n, ci = row % n, di = col / n, bi = col % n;
    if (bi == di) v = csub(v, a.P[(int64_t)ai * n + ci]);
    if (ai == ci) v = csub(v, a.Q[(int64_t)di * n + bi]);
    if (ai == ci && bi == di) v = cadd(v, make_double2(0.0, -(a.E[ai] - a.E[bi])));
    a.R[(int64_t)(ai * n + bi) * D + (ci * n + di)] = v;
  };
  gemm_tile(D, D, 2 * K, blockIdx.y * kTile, blockIdx.x * kTile, la, lb, epi);
}

// obs[r][o] = sum_ij E_o[j][i] rho_r[i][j]  (D-dot per observable and RHS)
__global__ void observe_kernel(int n, int R, int n_obs, const double2* Eops, const double2* P, double2* out) {
  const int64_t D = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)R * n_obs;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / n_obs), o = (int)(t % n_obs);
    double2 s = cz();
    for (int64_t e = 0; e < D; ++e) {
      const int i = (int)(e / n), j = (int)(e % n);
      cfma(s, Eops[o * D + (int64_t)j * n + i], P[e * R + r]);
    }
    out[(int64_t)r * n_obs + o] = s;
  }
}

}  // namespace rf
}  // namespace lime

using namespace lime;

extern "C" size_t lime_redfield_build_f64_workspace(int32_t n, int32_t k) {
  if (n <= 0 || k <= 0) return 0;
  const size_t nn = (size_t)n * n;
  return ((size_t)k * nn + 2 * nn) * sizeof(double2);
}

extern "C" int lime_redfield_build_f64(const LimeRedfieldBuildDesc* d, void* stream) {
  if (!d || d->n <= 0 || d->k <= 0 || d->spec_stride < 0) return LIME_ERR_ARG;
  if (!d->evals || !d->a_eig || !d->spec || !d->R || !d->workspace) return LIME_ERR_ARG;
  if ((int64_t)d->n * d->n > 46340) return LIME_ERR_UNSUPPORTED;   // D^2 must fit 31-bit tiles
  if (d->workspace_bytes < lime_redfield_build_f64_workspace(d->n, d->k)) return LIME_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const int n = d->n, k = d->k;
  const size_t nn = (size_t)n * n;
  double2* Lam = reinterpret_cast<double2*>(d->workspace);
  double2* P = Lam + (size_t)k * nn;
  double2* Q = P + nn;
  const double2* A = reinterpret_cast<const double2*>(d->a_eig);
  const int eb = (int)(((size_t)k * nn + 255) / 256);
  rf::lam_kernel<<<eb < 4096 ? eb : 4096, 256, 0, st>>>(n, k, A, d->spec, d->spec_stride, Lam);
  LIME_CUDA_TRY(cudaGetLastError());
  const int pb = (int)((nn + 255) / 256);
  rf::pq_kernel<<<pb, 256, 0, st>>>(n, k, A, Lam, P, Q);
  LIME_CUDA_TRY(cudaGetLastError());
  rf::BuildArgs a{n, k, d->evals, A, Lam, P, Q, reinterpret_cast<double2*>(d->R)};
  const int D = n * n;
  dim3 grid((D + rf::kTile - 1) / rf::kTile, (D + rf::kTile - 1) / rf::kTile);
  rf::assemble_kernel<<<grid, rf::kThreads, 0, st>>>(a);
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch(3);
  return LIME_OK;
}

extern "C" int lime_redfield_assemble_f64(const LimeRedfieldAssembleDesc* d, void* stream) {
  if (!d || d->n <= 0 || d->k <= 0) return LIME_ERR_ARG;
  if (!d->evals || !d->a_eig || !d->lam || !d->p || !d->q || !d->R) return LIME_ERR_ARG;
  if ((int64_t)d->n * d->n > 46340) return LIME_ERR_UNSUPPORTED;
  const int D = d->n * d->n;
  rf::BuildArgs a{d->n, d->k, d->evals, reinterpret_cast<const double2*>(d->a_eig),
                  reinterpret_cast<const double2*>(d->lam), reinterpret_cast<const double2*>(d->p),
                  reinterpret_cast<const double2*>(d->q), reinterpret_cast<double2*>(d->R)};
  dim3 grid((D + rf::kTile - 1) / rf::kTile, (D + rf::kTile - 1) / rf::kTile);
  rf::assemble_kernel<<<grid, rf::kThreads, 0, (cudaStream_t)stream>>>(a);
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch();
  return LIME_OK;
}

extern "C" size_t lime_redfield_rk4_f64_workspace(int32_t n, int32_t n_rhs) {
  if (n <= 0 || n_rhs <= 0) return 0;
  return (size_t)3 * n * n * n_rhs * sizeof(double2);
}

extern "C" int lime_redfield_rk4_f64(const LimeRedfieldRK4Desc* d, void* stream) {
  if (!d || d->n <= 0 || d->n_rhs <= 0 || d->n_steps < 0 || d->n_obs < 0) return LIME_ERR_ARG;
  if (!d->R || !d->rho || !d->workspace) return LIME_ERR_ARG;
  if (d->n_obs > 0 && (!d->obs_ops || !d->obs_out)) return LIME_ERR_ARG;
  if (d->states && d->states_every <= 0) return LIME_ERR_ARG;
  if ((int64_t)d->n * d->n > 46340) return LIME_ERR_UNSUPPORTED;
  if (d->workspace_bytes < lime_redfield_rk4_f64_workspace(d->n, d->n_rhs)) return LIME_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const int D = d->n * d->n, R = d->n_rhs;
  const size_t DR = (size_t)D * R;
  double2* P = reinterpret_cast<double2*>(d->rho);
  double2* acc = reinterpret_cast<double2*>(d->workspace);
  double2* S0 = acc + DR;
  double2* S1 = S0 + DR;
  const int obs_every = d->obs_every > 0 ? d->obs_every : 1;
  const int n_slots = d->n_steps / obs_every;
  dim3 grid((R + rf::kTile - 1) / rf::kTile, (D + rf::kTile - 1) / rf::kTile);
  int64_t launches = 0;
  for (int step = 0; step < d->n_steps; ++step) {
    const double2* S = P;
    for (int s = 0; s < 4; ++s) {
      double2* Sn = (s % 2 == 0) ? S0 : S1;
      rf::StageArgs a{D, R, s, d->dt, reinterpret_cast<const double2*>(d->R), S, P, acc, Sn};
      rf::stage_kernel<<<grid, rf::kThreads, 0, st>>>(a);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
      S = Sn;
    }
    if (d->n_obs > 0 && ((step + 1) % obs_every) == 0) {
      const int slot = (step + 1) / obs_every - 1;
      double2* tmp = reinterpret_cast<double2*>(d->obs_out);
      // obs_out layout [slot][R][n_obs]
      const int tb = (R * d->n_obs + 127) / 128;
      rf::observe_kernel<<<tb, 128, 0, st>>>(d->n, R, d->n_obs, reinterpret_cast<const double2*>(d->obs_ops), P,
                                             tmp + (size_t)slot * R * d->n_obs);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
    }
    if (d->states && ((step + 1) % d->states_every) == 0) {
      const int slot = (step + 1) / d->states_every - 1;
      LIME_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<double2*>(d->states) + (size_t)slot * DR, P,
                                    DR * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    }
    (void)n_slots;
  }
  count_launch(launches);
  return LIME_OK;
}
