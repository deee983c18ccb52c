// Gradients of the Bloch-Redfield path (no counterpart in the reference,
// which has no gradients; it differentiates redfield_tensor,
// lime/oqs.py:528-579, and the RK4 loop of _redfield, lime/oqs.py:453-472).
//
// 1. Adjoint of the generator assembly.  With the closed form
//      L[ab,cd] = -i (E_a - E_b) d_ac d_bd - d_bd P[a,c] - d_ac Q[d,b]
//                 + T[(a,c),(d,b)],   T = U V,
//      U[(a,c), k] = A_k[a,c],  U[(a,c), K+k] = Lam_k[a,c],
//      V[k, (d,b)] = conj(Lam_k[b,d]),  V[K+k, (d,b)] = A_k[d,b],
//    and G = dL/dconj(L) (the gradient of a real loss in torch's complex
//    convention, dl = Re sum conj(G) dL): grad_T = G permuted as
//    G'[(a,c),(d,b)] = G[ab,cd], grad_U = G' V^dag, grad_V = U^dag G' (two
//    FP64 GEMMs of the assembly's shape), grad_P[a,c] = -sum_b G[ab,cb],
//    grad_Q[d,b] = -sum_a G[ab,ad] and grad_E[a] = sum_b (Im G[ba,ba] -
//    Im G[ab,ab]).  The chain rule through Lam_k = C_k o A_k, P = sum A_k
//    Lam_k, Q = sum Lam_k^dag A_k, A_k = V^dag a_k V and eigh(H) (all
//    O(N^3 K) or smaller) is left to the caller.
//
// 2. Discrete adjoint of lime_redfield_rk4_f64 over one checkpoint segment,
//    for a block of right-hand sides: recompute the segment from its
//    checkpoint storing every stage input y_i, then walk the steps back:
//      lam += Et^dag g  (observables recorded after the step, Et = vec E^T)
//      a_4 = dt/6 lam;           yb_4 = L^dag a_4
//      a_3 = dt/3 lam + dt yb_4;  a_2 = dt/3 lam + dt/2 yb_3;  a_1 = dt/6 lam + dt/2 yb_2
//      lam <- lam + yb_4 + yb_3 + yb_2 + yb_1
//      grad_L += sum_i a_i y_i^dag          (one GEMM over the four stages)
//      grad_E[o][j][i] += g_o conj(rho[i][j])
//    FP64 throughout (the exact path; the tensor-core version is in
//    redfield_split.cu).

#include "gemm_f64.cuh"

namespace lime {
namespace rfa {

using rf::gemm_tile;
using rf::kThreads;
using rf::kTile;

// ---------------------------------------------------------------- assembly adjoint
struct AsmAdjArgs {
  int n, k;
  const double2* A;     // [k][n][n]
  const double2* Lam;   // [k][n][n]
  const double2* G;     // [D][D]
  double2* gA;          // [k][n][n]
  double2* gLam;        // [k][n][n]
};

// grad_U = G' V^dag: row (a,c), column kk; written over gA / gLam
__global__ void __launch_bounds__(kThreads) grad_u_kernel(AsmAdjArgs a) {
  const int n = a.n, K = a.k, D = n * n;
  const int64_t nn = (int64_t)n * n;
  auto la = [&](int row, int kd) -> double2 {          // G'[(a,c),(d,b)] = G[ab, cd]
    const int ai = row / n, ci = row % n, di = kd / n, bi = kd % n;
    return a.G[(int64_t)(ai * n + bi) * D + (ci * n + di)];
  };
  auto lb = [&](int kd, int kk) -> double2 {           // conj(V[kk, (d,b)])
    const int di = kd / n, bi = kd % n;
    return kk < K ? a.Lam[kk * nn + (int64_t)bi * n + di] : cconj(a.A[(kk - K) * nn + kd]);
  };
  auto epi = [&](int row, int kk, double2 v) {
    if (kk < K) a.gA[kk * nn + row] = v;
    else a.gLam[(kk - K) * nn + row] = v;
  };
  gemm_tile(D, 2 * K, D, blockIdx.y * kTile, blockIdx.x * kTile, la, lb, epi);
}

// grad_V = U^dag G': row kk, column (d,b); added to gLam / gA (after grad_u_kernel)
__global__ void __launch_bounds__(kThreads) grad_v_kernel(AsmAdjArgs a) {
  const int n = a.n, K = a.k, D = n * n;
  const int64_t nn = (int64_t)n * n;
  auto la = [&](int kk, int ac) -> double2 {           // conj(U[(a,c), kk])
    return cconj(kk < K ? a.A[kk * nn + ac] : a.Lam[(kk - K) * nn + ac]);
  };
  auto lb = [&](int ac, int db) -> double2 {
    const int ai = ac / n, ci = ac % n, di = db / n, bi = db % n;
    return a.G[(int64_t)(ai * n + bi) * D + (ci * n + di)];
  };
  auto epi = [&](int kk, int db, double2 v) {
    const int di = db / n, bi = db % n;
    if (kk < K) {   // V = conj(Lam[b,d]): grad_Lam[b,d] += conj(grad_V)
      double2& g = a.gLam[kk * nn + (int64_t)bi * n + di];
      g = cadd(g, cconj(v));
    } else {        // V = A[d,b]
      double2& g = a.gA[(kk - K) * nn + db];
      g = cadd(g, v);
    }
  };
  gemm_tile(2 * K, D, D, blockIdx.y * kTile, blockIdx.x * kTile, la, lb, epi);
}

// grad_P, grad_Q (n x n) and grad_E (n), one thread per (x, y)
__global__ void grad_local_kernel(int n, const double2* G, double2* gP, double2* gQ, double* gE) {
  const int D = n * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < D; e += gridDim.x * blockDim.x) {
    const int x = e / n, y = e % n;
    double2 p = cz(), q = cz();
    for (int m = 0; m < n; ++m) {
      p = csub(p, G[(int64_t)(x * n + m) * D + (y * n + m)]);   // -G[(x m),(y m)]: grad_P[x,y]
      q = csub(q, G[(int64_t)(m * n + y) * D + (m * n + x)]);   // -G[(m y),(m x)]: grad_Q[x,y]
    }
    gP[e] = p;
    gQ[e] = q;
    if (y == 0) {
      double s = 0.0;
      for (int b = 0; b < n; ++b)
        s += G[(int64_t)(b * n + x) * D + (b * n + x)].y - G[(int64_t)(x * n + b) * D + (x * n + b)].y;
      gE[x] = s;
    }
  }
}

// ---------------------------------------------------------------- RK4 adjoint
struct StepArgs {
  int D, R, n, n_obs;
  double dt;
  const double2* L;       // D x D
  double2* lam;           // D x R adjoint state
  double2* acc;           // D x R sum of yb of the step
  double2* a[4];          // adjoint stage inputs a_1..a_4, D x R each
  const double2* y[4];    // forward stage inputs y_1..y_4 of the step, D x R each
  double2* gL;            // D x D
};

// lam += Et^dag g and grad_E += g conj(rho) for the observables recorded
// after the step (rho = the state after it, D x R; Et[o][a n + b] = E_o[b][a]);
// then a_4 = dt/6 lam.  One thread per element of lam.
__global__ void source_kernel(StepArgs s, const double2* E, const double2* g, const double2* rho_after,
                              double2* gE) {
  const int D = s.D, R = s.R, n = s.n;
  const int64_t total = (int64_t)D * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int d = (int)(e / R), r = (int)(e % R);
    double2 l = s.lam[e];
    if (g != nullptr) {
      const int ai = d / n, bi = d % n;
      for (int o = 0; o < s.n_obs; ++o) {
        const double2 et = E[(int64_t)o * D + (int64_t)bi * n + ai];   // Et[o][d] = E_o[b][a]
        cfma(l, cconj(et), g[(int64_t)r * s.n_obs + o]);
      }
    }
    s.lam[e] = l;
    s.a[3][e] = cscale(l, s.dt / 6.0);
  }
  if (g != nullptr && gE != nullptr) {
    // grad_E[o][b][a] += sum_r g[r][o] conj(rho[(a,b)][r])
    const int64_t tot2 = (int64_t)s.n_obs * D;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot2; e += (int64_t)gridDim.x * blockDim.x) {
      const int o = (int)(e / D), d = (int)(e % D);
      const int ai = d / n, bi = d % n;
      double2 v = cz();
      for (int r = 0; r < R; ++r) cfma(v, g[(int64_t)r * s.n_obs + o], cconj(rho_after[(int64_t)d * R + r]));
      double2& t = gE[(int64_t)o * D + (int64_t)bi * n + ai];
      t = cadd(t, v);
    }
  }
}

// yb_i = L^dag a_i (i = stage 4, 3, 2, 1) with the adjoint combination fused:
// i > 1 writes a_{i-1}; i = 1 updates lam.
__global__ void __launch_bounds__(kThreads) adj_stage_kernel(StepArgs s, int i) {
  const int D = s.D, R = s.R;
  auto la = [&](int row, int k) -> double2 { return cconj(s.L[(int64_t)k * D + row]); };
  const double2* ain = s.a[i - 1];
  auto lb = [&](int k, int j) -> double2 { return ain[(int64_t)k * R + j]; };
  const double dt = s.dt;
  auto epi = [&](int row, int j, double2 yb) {
    const int64_t e = (int64_t)row * R + j;
    const double2 l = s.lam[e];
    if (i == 4) {
      s.acc[e] = yb;
      s.a[2][e] = cadd(cscale(l, dt / 3.0), cscale(yb, dt));
    } else if (i == 3) {
      s.acc[e] = cadd(s.acc[e], yb);
      s.a[1][e] = cadd(cscale(l, dt / 3.0), cscale(yb, dt / 2.0));
    } else if (i == 2) {
      s.acc[e] = cadd(s.acc[e], yb);
      s.a[0][e] = cadd(cscale(l, dt / 6.0), cscale(yb, dt / 2.0));
    } else {
      s.lam[e] = cadd(l, cadd(s.acc[e], yb));
    }
  };
  gemm_tile(D, R, D, blockIdx.y * kTile, blockIdx.x * kTile, la, lb, epi);
}

// grad_L += sum_i a_i y_i^dag: K = 4 R (stage, right-hand side)
__global__ void __launch_bounds__(kThreads) grad_l_kernel(StepArgs s) {
  const int D = s.D, R = s.R;
  auto la = [&](int row, int k) -> double2 { return s.a[k / R][(int64_t)row * R + k % R]; };
  auto lb = [&](int k, int col) -> double2 { return cconj(s.y[k / R][(int64_t)col * R + k % R]); };
  auto epi = [&](int row, int col, double2 v) {
    double2& g = s.gL[(int64_t)row * D + col];
    g = cadd(g, v);
  };
  gemm_tile(D, D, 4 * R, blockIdx.y * kTile, blockIdx.x * kTile, la, lb, epi);
}

}  // namespace rfa
}  // namespace lime

using namespace lime;
using rf::kThreads;
using rf::kTile;

extern "C" int lime_redfield_assemble_adjoint_f64(const LimeRedfieldAssembleAdjointDesc* d, void* stream) {
  if (!d || d->n <= 0 || d->k <= 0) return LIME_ERR_ARG;
  if (!d->a_eig || !d->lam || !d->G || !d->grad_evals || !d->grad_a || !d->grad_lam || !d->grad_p || !d->grad_q)
    return LIME_ERR_ARG;
  if ((int64_t)d->n * d->n > 46340) return LIME_ERR_UNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream;
  const int n = d->n, K = d->k, D = n * n;
  rfa::AsmAdjArgs a{n, K, reinterpret_cast<const double2*>(d->a_eig), reinterpret_cast<const double2*>(d->lam),
                    reinterpret_cast<const double2*>(d->G), reinterpret_cast<double2*>(d->grad_a),
                    reinterpret_cast<double2*>(d->grad_lam)};
  dim3 gu((2 * K + kTile - 1) / kTile, (D + kTile - 1) / kTile);
  rfa::grad_u_kernel<<<gu, kThreads, 0, st>>>(a);
  LIME_CUDA_TRY(cudaGetLastError());
  dim3 gv((D + kTile - 1) / kTile, (2 * K + kTile - 1) / kTile);
  rfa::grad_v_kernel<<<gv, kThreads, 0, st>>>(a);
  LIME_CUDA_TRY(cudaGetLastError());
  rfa::grad_local_kernel<<<(D + 255) / 256, 256, 0, st>>>(n, reinterpret_cast<const double2*>(d->G),
                                                         reinterpret_cast<double2*>(d->grad_p),
                                                         reinterpret_cast<double2*>(d->grad_q), d->grad_evals);
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch(3);
  return LIME_OK;
}

extern "C" size_t lime_redfield_adjoint_f64_workspace(int32_t n, int32_t n_rhs, int32_t seg_steps) {
  if (n <= 0 || n_rhs <= 0 || seg_steps <= 0) return 0;
  const size_t DR = (size_t)n * n * n_rhs * sizeof(double2);
  // stage inputs of the segment (4 per step) + the state after it, state,
  // RK4 accumulator, adjoint accumulator, adjoint stage inputs (4)
  return DR * (4 * (size_t)seg_steps + 1 + 2 + 1 + 4);
}

extern "C" int lime_redfield_adjoint_f64(const LimeRedfieldAdjointDesc* d, void* stream) {
  if (!d || d->n <= 0 || d->n_rhs <= 0 || d->seg_steps <= 0 || d->step0 < 0 || d->n_obs < 0) return LIME_ERR_ARG;
  if (!d->R || !d->ckpt || !d->lam || !d->grad_R || !d->workspace) return LIME_ERR_ARG;
  if (d->n_obs > 0 && (!d->obs_ops || !d->obs_grad)) return LIME_ERR_ARG;
  if ((int64_t)d->n * d->n > 46340) return LIME_ERR_UNSUPPORTED;
  if (d->workspace_bytes < lime_redfield_adjoint_f64_workspace(d->n, d->n_rhs, d->seg_steps)) return LIME_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  const int n = d->n, D = n * n, R = d->n_rhs, S = d->seg_steps;
  const size_t DR = (size_t)D * R;
  const int obs_every = d->obs_every > 0 ? d->obs_every : 1;
  double2* w = reinterpret_cast<double2*>(d->workspace);
  double2* ys = w;                          // [S][4][D][R]
  double2* after = ys + (size_t)S * 4 * DR; // state after the segment
  double2* P = after + DR;
  double2* racc = P + DR;
  double2* aacc = racc + DR;
  double2* ast = aacc + DR;                 // a_1..a_4
  const double2* L = reinterpret_cast<const double2*>(d->R);
  int64_t launches = 0;

  // ---- recompute the segment, storing the stage inputs y_1..y_4 of every step
  LIME_CUDA_TRY(cudaMemcpyAsync(P, d->ckpt, DR * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  LIME_CUDA_TRY(cudaMemcpyAsync(ys, d->ckpt, DR * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  dim3 grid((R + kTile - 1) / kTile, (D + kTile - 1) / kTile);
  for (int step = 0; step < S; ++step) {
    double2* y = ys + (size_t)step * 4 * DR;
    for (int s = 0; s < 4; ++s) {
      double2* Sn = s < 3 ? y + (size_t)(s + 1) * DR : (step + 1 < S ? ys + (size_t)(step + 1) * 4 * DR : after);
      rf::StageArgs a{D, R, s, d->dt, L, y + (size_t)s * DR, P, racc, Sn};
      rf::stage_kernel<<<grid, kThreads, 0, st>>>(a);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
    }
  }

  // ---- backward over the steps of the segment
  rfa::StepArgs sa{};
  sa.D = D; sa.R = R; sa.n = n; sa.n_obs = d->n_obs; sa.dt = d->dt;
  sa.L = L;
  sa.lam = reinterpret_cast<double2*>(d->lam);
  sa.acc = aacc;
  for (int i = 0; i < 4; ++i) sa.a[i] = ast + (size_t)i * DR;
  sa.gL = reinterpret_cast<double2*>(d->grad_R);
  const int eb = (int)((DR + 255) / 256 < 65535 ? (DR + 255) / 256 : 65535);
  const int n_slots_total = d->n_slots;
  for (int step = S - 1; step >= 0; --step) {
    const int gstep = d->step0 + step;
    const double2* g = nullptr;
    if (d->n_obs > 0 && ((gstep + 1) % obs_every) == 0) {
      const int slot = (gstep + 1) / obs_every - 1;
      if (slot < n_slots_total)
        g = reinterpret_cast<const double2*>(d->obs_grad) + (size_t)slot * R * d->n_obs;
    }
    const double2* rho_after = step + 1 < S ? ys + (size_t)(step + 1) * 4 * DR : after;
    rfa::source_kernel<<<eb, 256, 0, st>>>(sa, reinterpret_cast<const double2*>(d->obs_ops), g, rho_after,
                                           reinterpret_cast<double2*>(d->grad_obs));
    LIME_CUDA_TRY(cudaGetLastError());
    ++launches;
    for (int i = 0; i < 4; ++i) sa.y[i] = ys + ((size_t)step * 4 + i) * DR;
    for (int i = 4; i >= 1; --i) {
      rfa::adj_stage_kernel<<<grid, kThreads, 0, st>>>(sa, i);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
    }
    dim3 gg((D + kTile - 1) / kTile, (D + kTile - 1) / kTile);
    rfa::grad_l_kernel<<<gg, kThreads, 0, st>>>(sa);
    LIME_CUDA_TRY(cudaGetLastError());
    ++launches;
  }
  count_launch(launches);
  return LIME_OK;
}
