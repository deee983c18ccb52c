// Plain FP64 Lindblad RK4 propagator (sm_103a).
//
// One CTA owns one density matrix for the whole time loop: every RK4 stage is
// a CTA-wide complex GEMM X = Heff * rho_s (register-tiled, operands staged
// through shared memory) followed by a fused epilogue that forms
//   f = -i (X - X^dag) + M o rho_s + sum_k L_k rho_s L_k^dag
// and the RK4 stage combination (lime/phys.py:636-649), then the trace check
// and the observables of lime/phys.py:837-844.  rho is Hermitian (the host
// splits non-Hermitian inputs), so rho Heff^dag = (Heff rho)^dag and one GEMM
// per stage gives the whole coherent + anti-Hermitian part.
//
// GB300 executes FP64 at a small fraction of its tensor rate, so this path is
// DFMA-bound for every size; its job is to be exact (it is the GPU FP64
// reference for the split-precision propagator), not fast.

#include "common.cuh"

namespace lime {
namespace f64 {

constexpr int kThreads = 256;
constexpr int kKC = 16;  // k-chunk of the shared-memory tiles

// Workspace layout per instance (complex elements): rs | X | acc | [Y | J] | Heff(t)
__host__ __device__ inline int64_t ws_mats(int k_dense) { return k_dense > 0 ? 6 : 4; }

// C (+)= A * op(B), all n x n, row-major, global memory; whole CTA.
// op(B) = B (conjb = false) or B^dag (conjb = true).
template <int TM>
__device__ void cta_cgemm(const double2* __restrict__ A, const double2* __restrict__ B,
                          bool conjb, double2* __restrict__ C, bool accumulate, int n,
                          double2* smem) {
  constexpr int T = 16 * TM;
  double2* As = smem;                   // [T][kKC + 1]
  double2* Bs = smem + T * (kKC + 1);   // [kKC][T + 1]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int i0 = 0; i0 < n; i0 += T) {
    for (int j0 = 0; j0 < n; j0 += T) {
      double2 acc[TM][TM];
#pragma unroll
      for (int u = 0; u < TM; ++u)
#pragma unroll
        for (int v = 0; v < TM; ++v) acc[u][v] = cz();
      for (int k0 = 0; k0 < n; k0 += kKC) {
        for (int idx = threadIdx.x; idx < T * kKC; idx += kThreads) {
          const int r = idx / kKC, c = idx % kKC;
          const int gi = i0 + r, gk = k0 + c;
          As[r * (kKC + 1) + c] = (gi < n && gk < n) ? A[(int64_t)gi * n + gk] : cz();
        }
        if (!conjb) {
          for (int idx = threadIdx.x; idx < T * kKC; idx += kThreads) {
            const int r = idx / T, c = idx % T;
            const int gk = k0 + r, gj = j0 + c;
            Bs[r * (T + 1) + c] = (gk < n && gj < n) ? B[(int64_t)gk * n + gj] : cz();
          }
        } else {
          // op(B)[k][j] = conj(B[j][k]); read along k for coalescing
          for (int idx = threadIdx.x; idx < T * kKC; idx += kThreads) {
            const int c = idx / kKC, r = idx % kKC;
            const int gk = k0 + r, gj = j0 + c;
            Bs[r * (T + 1) + c] = (gk < n && gj < n) ? cconj(B[(int64_t)gj * n + gk]) : cz();
          }
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kKC; ++kk) {
          double2 a[TM], b[TM];
#pragma unroll
          for (int u = 0; u < TM; ++u) a[u] = As[(ty + 16 * u) * (kKC + 1) + kk];
#pragma unroll
          for (int v = 0; v < TM; ++v) b[v] = Bs[kk * (T + 1) + tx + 16 * v];
#pragma unroll
          for (int u = 0; u < TM; ++u)
#pragma unroll
            for (int v = 0; v < TM; ++v) cfma(acc[u][v], a[u], b[v]);
        }
        __syncthreads();
      }
#pragma unroll
      for (int u = 0; u < TM; ++u) {
#pragma unroll
        for (int v = 0; v < TM; ++v) {
          const int gi = i0 + ty + 16 * u, gj = j0 + tx + 16 * v;
          if (gi < n && gj < n) {
            double2* c = C + (int64_t)gi * n + gj;
            *c = accumulate ? cadd(*c, acc[u][v]) : acc[u][v];
          }
        }
      }
    }
  }
  __syncthreads();
}

struct RK4Args {
  int n, param_batch, n_steps, k_dense, n_obs, obs_diag, states_every, states_per_inst, step0;
  double dt, trace_tol;
  double2* rho;
  const double2* heff;    int64_t heff_stride;
  const double2* m;       int64_t m_stride;
  const double2* l_dense; int64_t l_dense_stride;
  const double2* obs_ops; int64_t obs_stride;
  double2* obs_out;       int obs_every, obs_per_inst;
  double2* states;
  double2* ws;
  double* tr0;
  int32_t* status;
  int n_drive;
  const double2* drive_ops;
  const double* drive_coef;
  // extents for the bounds-checked build (elements of obs_out and states)
  size_t obs_elems = kNoExtent, states_elems = kNoExtent;
};

template <int TM>
__global__ void __launch_bounds__(kThreads) lindblad_rk4_f64_kernel(RK4Args a) {
  extern __shared__ double2 smem[];
  __shared__ double red[kThreads / 32];
  const int b = blockIdx.x;
  const int n = a.n;
  const int64_t nn = (int64_t)n * n;
  const int p = b % a.param_batch;
  double2* rho = a.rho + b * nn;
  const double2* heff0 = a.heff + p * a.heff_stride;
  const double2* m = a.m ? a.m + p * a.m_stride : nullptr;
  const double2* ld = a.l_dense ? a.l_dense + p * a.l_dense_stride : nullptr;
  const double2* obs_ops = a.obs_ops ? a.obs_ops + p * a.obs_stride : nullptr;
  double2* ws = a.ws + (int64_t)b * ws_mats(a.k_dense) * nn;
  double2* rs = ws;
  double2* X = ws + nn;
  double2* acc = ws + 2 * nn;
  double2* Y = ws + 3 * nn;
  double2* J = ws + 4 * nn;
  double2* heff_t = ws + (ws_mats(a.k_dense) - 1) * nn;

  // trace at the start of the call (first chunk) for the drift check
  if (a.step0 == 0) {
    double t = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) t += rho[(int64_t)i * n + i].x;
    t = block_sum<kThreads>(t, red);
    if (threadIdx.x == 0) a.tr0[b] = t;
  }
  for (int64_t e = threadIdx.x; e < nn; e += kThreads) rs[e] = rho[e];
  __syncthreads();
  const double tr0 = a.tr0[b];

  const double dt = a.dt, dt2 = a.dt / 2.0;
  int flags = 0;
  for (int step = 0; step < a.n_steps; ++step) {
    // driven generator (lime/oqs.py:1716-1722): Heff(t) = Heff0 - sum_i f_i(t) H_i
    // with f_i evaluated at the end of the step
    const double2* heff = heff0;
    if (a.n_drive > 0) {
      const double* c = a.drive_coef + (int64_t)(a.step0 + step) * a.n_drive;
      for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
        double2 v = heff0[e];
        for (int q = 0; q < a.n_drive; ++q) v = csub(v, cscale(a.drive_ops[q * nn + e], c[q]));
        heff_t[e] = v;
      }
      __syncthreads();
      heff = heff_t;
    }
#pragma unroll 1
    for (int s = 0; s < 4; ++s) {
      cta_cgemm<TM>(heff, rs, false, X, false, n, smem);
      for (int k = 0; k < a.k_dense; ++k) {
        const double2* L = ld + k * nn;
        cta_cgemm<TM>(L, rs, false, Y, false, n, smem);
        cta_cgemm<TM>(Y, L, true, J, k > 0, n, smem);
      }
      const double cstage = (s == 2) ? dt : dt2;
      for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
        const int i = (int)(e / n), j = (int)(e % n);
        const double2 x = X[e], xt = X[(int64_t)j * n + i];
        // -i (x - conj(xt))
        const double2 d = make_double2(x.x - xt.x, x.y + xt.y);
        double2 f = make_double2(d.y, -d.x);
        const double2 r = rs[e];
        if (m) f = cadd(f, cmul(m[e], r));
        if (a.k_dense > 0) f = cadd(f, J[e]);
        if (s == 0) {
          acc[e] = f;
          rs[e] = cadd(rho[e], cscale(f, cstage));
        } else if (s < 3) {
          acc[e] = cadd(acc[e], cscale(f, 2.0));
          rs[e] = cadd(rho[e], cscale(f, cstage));
        } else {
          const double2 sum = cadd(acc[e], f);
          const double2 nr = cadd(rho[e], cscale(make_double2(sum.x / 6., sum.y / 6.), dt));
          rho[e] = nr;
          rs[e] = nr;
          if (!cfinite(nr)) flags |= LIME_FLAG_NONFINITE;
        }
      }
      __syncthreads();
    }
    // observables after the step
    const int gstep = a.step0 + step;
    const bool obs_now = ((gstep + 1) % a.obs_every) == 0;
    const int oslot = (gstep + 1) / a.obs_every - 1;
    for (int o = 0; obs_now && o < a.n_obs; ++o) {
      double sr = 0.0, si = 0.0;
      if (a.obs_diag) {
        const double2* E = obs_ops + (int64_t)o * n;
        for (int i = threadIdx.x; i < n; i += kThreads) {
          const double2 p = cmul(E[i], rho[(int64_t)i * n + i]);
          sr += p.x; si += p.y;
        }
      } else {
        const double2* E = obs_ops + o * nn;
        for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
          const int i = (int)(e / n), j = (int)(e % n);
          const double2 p = cmul(E[(int64_t)j * n + i], rho[e]);
          sr += p.x; si += p.y;
        }
      }
      sr = block_sum<kThreads>(sr, red);
      si = block_sum<kThreads>(si, red);
      const size_t oi = ((size_t)b * a.obs_per_inst + oslot) * a.n_obs + o;
      if (threadIdx.x == 0 && in_bounds(oi * 16, 16, a.obs_elems * 16, a.status))
        a.obs_out[oi] = make_double2(sr, si);
    }
    if (a.trace_tol > 0.0) {
      double t = 0.0;
      for (int i = threadIdx.x; i < n; i += kThreads) t += rho[(int64_t)i * n + i].x;
      t = block_sum<kThreads>(t, red);
      if (fabs(t - tr0) > a.trace_tol * fmax(1.0, fabs(tr0))) flags |= LIME_FLAG_TRACE_DRIFT;
    }
    if (a.states && ((gstep + 1) % a.states_every) == 0) {
      const int slot = (gstep + 1) / a.states_every - 1;
      double2* dst = a.states + ((int64_t)b * a.states_per_inst + slot) * nn;
      if (in_bounds((((size_t)b * a.states_per_inst + slot) * nn) * 16, (size_t)nn * 16, a.states_elems * 16,
                    a.status))
        for (int64_t e = threadIdx.x; e < nn; e += kThreads) dst[e] = rho[e];
    }
  }
  if (flags) atomicOr(a.status, flags);
}

// ---------------------------------------------------------------- adjoint
// One generator in the Hermitian form f = -i(G x - x G^dag) + M o x + sum_k L_k x L_k^dag.
struct Gen {
  const double2* g;
  const double2* m;   // may be null
  const double2* l;   // k dense operators, may be null
  int k;
};

// out = gen(x); X, Y, J are n x n scratch.  Whole CTA; ends synchronised.
template <int TM>
__device__ void apply_gen(const Gen& G, const double2* x, double2* out, double2* X, double2* Y, double2* J, int n,
                          double2* smem) {
  const int64_t nn = (int64_t)n * n;
  cta_cgemm<TM>(G.g, x, false, X, false, n, smem);
  for (int k = 0; k < G.k; ++k) {
    const double2* L = G.l + k * nn;
    cta_cgemm<TM>(L, x, false, Y, false, n, smem);
    cta_cgemm<TM>(Y, L, true, J, k > 0, n, smem);
  }
  for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
    const int i = (int)(e / n), j = (int)(e % n);
    const double2 a = X[e], b = X[(int64_t)j * n + i];
    double2 f = make_double2(a.y + b.y, b.x - a.x);   // -i (X - X^dag)
    if (G.m) f = cadd(f, cmul(G.m[e], x[e]));
    if (G.k > 0) f = cadd(f, J[e]);
    out[e] = f;
  }
  __syncthreads();
}

struct AdjArgs {
  int n, param_batch, seg_steps, step0, total_steps, k_dense, n_obs, obs_diag, obs_every, obs_per_inst;
  double dt;
  const double2* ckpt;
  double2* lam;
  const double2* heff; int64_t heff_stride;
  const double2* m; int64_t m_stride;
  const double2* ld; int64_t ld_stride;
  const double2* heff_adj; int64_t heff_adj_stride;
  const double2* m_adj; int64_t m_adj_stride;
  const double2* ld_adj; int64_t ld_adj_stride;
  const double2* obs_ops; int64_t obs_stride;
  const double2* obs_grad;
  double* g_diag;
  double* g_bond;
  double* g_gamma;
  double2* ws;
};

__host__ __device__ inline int64_t adj_ws_mats(int seg_steps, int k_dense) {
  return (int64_t)seg_steps + 9 + (k_dense > 0 ? 2 : 0);
}

// Parameter-gradient contributions of one stage: abar = adjoint of the stage
// derivative, y = stage state (both Hermitian).  Thread-strided over rows.
__device__ void grad_terms(const double2* abar, const double2* y, int n, double* gd, double* gb, double* gg) {
  for (int k = threadIdx.x; k < n; k += kThreads) {
    double sd = 0.0, sg = 0.0, sb = 0.0;
    for (int x = 0; x < n; ++x) {
      const double2 a = abar[(int64_t)k * n + x], v = y[(int64_t)k * n + x];
      sd += a.x * v.y - a.y * v.x;                 // Im(conj(a) y)
      if (x != k) sg -= a.x * v.x + a.y * v.y;      // -Re(conj(a) y), off-diagonal
      if (k + 1 < n) {
        const double2 a2 = abar[(int64_t)(k + 1) * n + x], v2 = y[(int64_t)(k + 1) * n + x];
        sb += (a.x * v2.y - a.y * v2.x) + (a2.x * v.y - a2.y * v.x);
      }
    }
    gd[k] += 2.0 * sd;
    gg[k] += sg;
    if (k + 1 < n) gb[k] += 2.0 * sb;
  }
}

template <int TM>
__global__ void __launch_bounds__(kThreads) lindblad_adjoint_f64_kernel(AdjArgs a) {
  extern __shared__ double2 smem[];
  const int b = blockIdx.x;
  const int n = a.n;
  const int64_t nn = (int64_t)n * n;
  const int p = b % a.param_batch;
  const Gen F{a.heff + p * a.heff_stride, a.m ? a.m + p * a.m_stride : nullptr,
              a.ld ? a.ld + p * a.ld_stride : nullptr, a.k_dense};
  const Gen A{a.heff_adj + p * a.heff_adj_stride, a.m_adj ? a.m_adj + p * a.m_adj_stride : nullptr,
              a.ld_adj ? a.ld_adj + p * a.ld_adj_stride : nullptr, a.k_dense};
  double2* ws = a.ws + (int64_t)b * adj_ws_mats(a.seg_steps, a.k_dense) * nn;
  double2* seg = ws;                              // rho_{step0 + s}, s < seg_steps
  double2* y2 = ws + (int64_t)a.seg_steps * nn;
  double2* y3 = y2 + nn;
  double2* y4 = y3 + nn;
  double2* kk = y4 + nn;
  double2* ab = kk + nn;
  double2* yb = ab + nn;
  double2* lnew = yb + nn;
  double2* X = lnew + nn;
  double2* lam_s = X + nn;
  double2* Y = lam_s + nn;
  double2* J = Y + nn;
  double2* lam = a.lam + (int64_t)b * nn;
  const double2* obs_ops = a.obs_ops ? a.obs_ops + p * a.obs_stride : nullptr;
  const double dt = a.dt, dt2 = a.dt / 2.0;

  // ---- forward recompute of the segment from its checkpoint ----
  for (int64_t e = threadIdx.x; e < nn; e += kThreads) seg[e] = a.ckpt[(int64_t)b * nn + e];
  __syncthreads();
  for (int s = 0; s + 1 < a.seg_steps; ++s) {
    const double2* r = seg + (int64_t)s * nn;
    double2* nxt = seg + (int64_t)(s + 1) * nn;
    // nxt accumulates k1 + 2k2 + 2k3 + k4 ; y2 holds the current stage input
    apply_gen<TM>(F, r, kk, X, Y, J, n, smem);
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) { nxt[e] = kk[e]; y2[e] = cadd(r[e], cscale(kk[e], dt2)); }
    __syncthreads();
    apply_gen<TM>(F, y2, kk, X, Y, J, n, smem);
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) { nxt[e] = cadd(nxt[e], cscale(kk[e], 2.0)); y2[e] = cadd(r[e], cscale(kk[e], dt2)); }
    __syncthreads();
    apply_gen<TM>(F, y2, kk, X, Y, J, n, smem);
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) { nxt[e] = cadd(nxt[e], cscale(kk[e], 2.0)); y2[e] = cadd(r[e], cscale(kk[e], dt)); }
    __syncthreads();
    apply_gen<TM>(F, y2, kk, X, Y, J, n, smem);
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
      const double2 sum = cadd(nxt[e], kk[e]);
      nxt[e] = cadd(r[e], cscale(make_double2(sum.x / 6., sum.y / 6.), dt));
    }
    __syncthreads();
  }

  // ---- backward through the segment ----
  double* GD = a.g_diag + (int64_t)b * n;
  double* GB = a.g_bond + (int64_t)b * (n > 1 ? n - 1 : 1);
  double* GG = a.g_gamma + (int64_t)b * n;
  for (int s = a.seg_steps - 1; s >= 0; --s) {
    const int gstep = a.step0 + s;   // the step rho_{gstep} -> rho_{gstep+1}
    // source: observable recorded after this step, Tr(E rho_{gstep+1})
    if (a.n_obs > 0 && ((gstep + 1) % a.obs_every) == 0) {
      const int slot = (gstep + 1) / a.obs_every - 1;
      const double2* gr = a.obs_grad + ((int64_t)b * a.obs_per_inst + slot) * a.n_obs;
      for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
        const int i = (int)(e / n), j = (int)(e % n);
        double2 add = cz();
        for (int o = 0; o < a.n_obs; ++o) {
          // Hermitian part of g E^dag: (g conj(E_ji) + conj(g) E_ij) / 2
          double2 eji, eij;
          if (a.obs_diag) {
            const double2 d = (i == j) ? obs_ops[(int64_t)o * n + i] : cz();
            eji = d; eij = d;
          } else {
            eji = obs_ops[o * nn + (int64_t)j * n + i];
            eij = obs_ops[o * nn + (int64_t)i * n + j];
          }
          const double2 g = gr[o];
          add = cadd(add, cscale(cadd(cmul(g, cconj(eji)), cmul(cconj(g), eij)), 0.5));
        }
        lam[e] = cadd(lam[e], add);
      }
      __syncthreads();
    }
    const double2* r = seg + (int64_t)s * nn;
    // stage states y2, y3, y4 (y1 = r)
    apply_gen<TM>(F, r, kk, X, Y, J, n, smem);
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) y2[e] = cadd(r[e], cscale(kk[e], dt2));
    __syncthreads();
    apply_gen<TM>(F, y2, kk, X, Y, J, n, smem);
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) y3[e] = cadd(r[e], cscale(kk[e], dt2));
    __syncthreads();
    apply_gen<TM>(F, y3, kk, X, Y, J, n, smem);
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) y4[e] = cadd(r[e], cscale(kk[e], dt));
    __syncthreads();
    // adjoint stages
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
      lam_s[e] = lam[e];
      ab[e] = cscale(lam[e], dt / 6.0);
    }
    __syncthreads();
    apply_gen<TM>(A, ab, yb, X, Y, J, n, smem);                   // ybar4
    grad_terms(ab, y4, n, GD, GB, GG);
    __syncthreads();
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
      lnew[e] = cadd(lam_s[e], yb[e]);
      ab[e] = cadd(cscale(lam_s[e], dt / 3.0), cscale(yb[e], dt));
    }
    __syncthreads();
    apply_gen<TM>(A, ab, yb, X, Y, J, n, smem);                   // ybar3
    grad_terms(ab, y3, n, GD, GB, GG);
    __syncthreads();
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
      lnew[e] = cadd(lnew[e], yb[e]);
      ab[e] = cadd(cscale(lam_s[e], dt / 3.0), cscale(yb[e], dt2));
    }
    __syncthreads();
    apply_gen<TM>(A, ab, yb, X, Y, J, n, smem);                   // ybar2
    grad_terms(ab, y2, n, GD, GB, GG);
    __syncthreads();
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) {
      lnew[e] = cadd(lnew[e], yb[e]);
      ab[e] = cadd(cscale(lam_s[e], dt / 6.0), cscale(yb[e], dt2));
    }
    __syncthreads();
    apply_gen<TM>(A, ab, yb, X, Y, J, n, smem);                   // ybar1
    grad_terms(ab, r, n, GD, GB, GG);
    __syncthreads();
    for (int64_t e = threadIdx.x; e < nn; e += kThreads) lam[e] = cadd(lnew[e], yb[e]);
    __syncthreads();
  }
}

// Heff = H - (i/2) sum_k L_k^dag L_k ;  M = sum_k l_k l_k^dag, one CTA per
// generator.  The dense part sum_k L_k^dag L_k arrives in heff (a strided
// batched GEMM run before this kernel) or is absent (k_dense = 0).  For the
// diagonal operators the diagonal sums dg[i] = sum_k |l_k[i]|^2 (which are
// both the diagonal of sum_k L_k^dag L_k and of M) are formed once per
// generator in shared memory, k in order, then the site-dephasing rate r_i;
// when every diagonal operator has at most one nonzero entry (site
// dephasing) the off-diagonal terms l_k[i] conj(l_k[j]) of M are exact zeros
// and are not summed.
__global__ void __launch_bounds__(kThreads) prepare_kernel(LimePrepareDesc d) {
  extern __shared__ double dg[];    // [n]
  const int b = blockIdx.x;
  const int n = d.n;
  const int nn = n * n;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const double2* H = reinterpret_cast<const double2*>(d.h) + b * d.h_stride;
  const double2* lg = d.l_diag ? reinterpret_cast<const double2*>(d.l_diag) + b * d.l_diag_stride : nullptr;
  const double* rate = d.dephasing ? d.dephasing + b * d.dephasing_stride : nullptr;
  double2* heff = reinterpret_cast<double2*>(d.heff) + (int64_t)b * nn;
  double2* M = reinterpret_cast<double2*>(d.m) + (int64_t)b * nn;
  __shared__ int spread;   // some l_k has two or more nonzero entries
  if (t == 0) spread = 0;
  for (int i = t; i < n; i += kThreads) {
    double s = 0.0;
    for (int k = 0; k < d.k_diag; ++k) {
      const double2 v = lg[(int64_t)k * n + i];
      s += v.x * v.x + v.y * v.y;
    }
    dg[i] = rate ? s + rate[i] : s;
  }
  __syncthreads();
  // one warp per operator counts its nonzero entries
  for (int k = warp; k < d.k_diag; k += kThreads / 32) {
    int cnt = 0;
    for (int i0 = 0; i0 < n; i0 += 32) {   // every lane takes part in each ballot
      const int i = i0 + lane;
      const double2 v = i < n ? lg[(int64_t)k * n + i] : cz();
      cnt += __popc(__ballot_sync(0xffffffffu, v.x != 0.0 || v.y != 0.0));
    }
    if (lane == 0 && cnt > 1) atomicOr(&spread, 1);
  }
  __syncthreads();
  for (int e = t; e < nn; e += kThreads) {
    const int i = e / n, j = e - i * n;
    double2 g = d.k_dense > 0 ? heff[e] : cz();   // (sum_k L_k^dag L_k)_ij of the dense operators
    double2 mm = cz();
    if (i == j) {
      g.x += dg[i];
      mm.x = dg[i];
    } else if (spread) {
      for (int k = 0; k < d.k_diag; ++k) {
        const double2* l = lg + (int64_t)k * n;
        cfma(mm, l[i], cconj(l[j]));
      }
    }
    // H - (i/2) g  =  (H.re + g.im/2, H.im - g.re/2)
    const double2 h = H[e];
    heff[e] = make_double2(h.x + 0.5 * g.y, h.y - 0.5 * g.x);
    M[e] = mm;
  }
}

}  // namespace f64
}  // namespace lime

using namespace lime;

extern "C" int lime_lindblad_prepare_f64(const LimePrepareDesc* d, void* stream) {
  if (!d || d->n <= 0 || d->batch <= 0 || d->k_dense < 0 || d->k_diag < 0) return LIME_ERR_ARG;
  if (!d->h || !d->heff || !d->m) return LIME_ERR_ARG;
  if ((d->k_dense > 0 && !d->l_dense) || (d->k_diag > 0 && !d->l_diag)) return LIME_ERR_ARG;
  if (d->h_stride < 0 || d->l_dense_stride < 0 || d->l_diag_stride < 0 || d->dephasing_stride < 0)
    return LIME_ERR_ARG;
  if ((size_t)d->n * sizeof(double) > 48 * 1024) return LIME_ERR_UNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream;
  if (d->k_dense > 0) {
    // heff[b] = sum_k L_k^dag L_k = [L_1; ..; L_K]^dag [L_1; ..; L_K] (K n x n
    // stacked), one strided batched FP64 GEMM over the generators
    LimeZgemmDesc g{};
    const int64_t n = d->n;
    g.M = d->n; g.N = d->n; g.K = (int32_t)(d->k_dense * n); g.batch = d->batch;
    g.conj_a = 1;
    g.A = d->l_dense; g.a_rs = 1; g.a_cs = n; g.a_bs = d->l_dense_stride;
    g.B = d->l_dense; g.b_rs = n; g.b_cs = 1; g.b_bs = d->l_dense_stride;
    g.C = d->heff; g.c_rs = n; g.c_cs = 1; g.c_bs = n * n;
    const int rc = lime_zgemm_strided_f64(&g, stream);
    if (rc != LIME_OK) return rc;
  }
  f64::prepare_kernel<<<d->batch, f64::kThreads, (size_t)d->n * sizeof(double), st>>>(*d);
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch();
  return LIME_OK;
}

extern "C" size_t lime_lindblad_rk4_f64_workspace(int32_t n, int32_t batch, int32_t k_dense) {
  if (n <= 0 || batch <= 0 || k_dense < 0) return 0;
  const size_t mats = (size_t)f64::ws_mats(k_dense) * (size_t)n * n * sizeof(double2);
  return (size_t)batch * (mats + sizeof(double));
}

template <int TM>
static int launch_f64(f64::RK4Args& args, int batch, cudaStream_t st) {
  const size_t smem = (size_t)(16 * TM) * (f64::kKC + 1) * sizeof(double2) +
                      (size_t)f64::kKC * (16 * TM + 1) * sizeof(double2);
  auto kern = f64::lindblad_rk4_f64_kernel<TM>;
  LIME_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<batch, f64::kThreads, smem, st>>>(args);
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch();
  return LIME_OK;
}

extern "C" int lime_lindblad_rk4_f64(const LimeLindbladDesc* d, void* stream) {
  if (!d) return LIME_ERR_ARG;
  if (d->n <= 0 || d->batch <= 0 || d->n_steps < 0 || d->k_dense < 0 || d->n_obs < 0) return LIME_ERR_ARG;
  if (!d->rho || !d->heff || !d->status || !d->workspace) return LIME_ERR_ARG;
  if (d->k_dense > 0 && !d->l_dense) return LIME_ERR_ARG;
  if (d->n_obs > 0 && (!d->obs_ops || !d->obs_out)) return LIME_ERR_ARG;
  if (d->states && d->states_every <= 0) return LIME_ERR_ARG;
  if (d->heff_stride < 0 || d->m_stride < 0 || d->l_dense_stride < 0 || d->obs_stride < 0) return LIME_ERR_ARG;
  const int pb = d->param_batch > 0 ? d->param_batch : d->batch;
  if (pb > d->batch) return LIME_ERR_ARG;
  if (!(d->dt == d->dt)) return LIME_ERR_ARG;
  if (d->n_drive < 0 || (d->n_drive > 0 && (!d->drive_ops || !d->drive_coef))) return LIME_ERR_ARG;
  if (d->workspace_bytes < lime_lindblad_rk4_f64_workspace(d->n, d->batch, d->k_dense))
    return LIME_ERR_WORKSPACE;
  if (d->n_steps == 0) return LIME_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nn = (int64_t)d->n * d->n;
  f64::RK4Args a{};
  a.n = d->n; a.param_batch = pb; a.k_dense = d->k_dense; a.n_obs = d->n_obs; a.obs_diag = d->obs_diag;
  a.states_every = d->states ? d->states_every : 1;
  a.states_per_inst = d->states ? d->n_steps / d->states_every : 0;
  a.dt = d->dt; a.trace_tol = d->trace_tol;
  a.rho = reinterpret_cast<double2*>(d->rho);
  a.heff = reinterpret_cast<const double2*>(d->heff); a.heff_stride = d->heff_stride;
  a.m = reinterpret_cast<const double2*>(d->m); a.m_stride = d->m_stride;
  a.l_dense = reinterpret_cast<const double2*>(d->l_dense); a.l_dense_stride = d->l_dense_stride;
  a.obs_ops = reinterpret_cast<const double2*>(d->obs_ops); a.obs_stride = d->obs_stride;
  a.obs_out = reinterpret_cast<double2*>(d->obs_out);
  a.obs_every = d->obs_every > 0 ? d->obs_every : 1;
  a.obs_per_inst = d->n_steps / a.obs_every;
  a.states = reinterpret_cast<double2*>(d->states);
  a.obs_elems = (size_t)d->batch * a.obs_per_inst * (d->n_obs > 0 ? d->n_obs : 0);
  a.states_elems = (size_t)d->batch * a.states_per_inst * nn;
  a.ws = reinterpret_cast<double2*>(d->workspace);
  a.tr0 = reinterpret_cast<double*>(reinterpret_cast<char*>(d->workspace) +
                                    (size_t)d->batch * f64::ws_mats(d->k_dense) * nn * sizeof(double2));
  a.status = d->status;
  a.n_drive = d->n_drive;
  a.drive_ops = reinterpret_cast<const double2*>(d->drive_ops);
  a.drive_coef = d->drive_coef;
  // bounded launches: at most ~2^27 complex MACs of GEMM per instance per launch
  const double per_step = 4.0 * (1 + 2 * d->k_dense) * (double)nn * d->n;
  int chunk = (int)fmax(1.0, fmin((double)d->n_steps, 134217728.0 / per_step));
  for (int s0 = 0; s0 < d->n_steps; s0 += chunk) {
    a.step0 = s0;
    a.n_steps = (d->n_steps - s0 < chunk) ? d->n_steps - s0 : chunk;
    int rc;
    if (d->n <= 16) rc = launch_f64<1>(a, d->batch, st);
    else if (d->n <= 32) rc = launch_f64<2>(a, d->batch, st);
    else rc = launch_f64<4>(a, d->batch, st);
    if (rc != LIME_OK) return rc;
  }
  return LIME_OK;
}

extern "C" size_t lime_lindblad_adjoint_f64_workspace(int32_t n, int32_t batch, int32_t seg_steps, int32_t k_dense) {
  if (n <= 0 || batch <= 0 || seg_steps <= 0 || k_dense < 0) return 0;
  return (size_t)batch * (size_t)f64::adj_ws_mats(seg_steps, k_dense) * (size_t)n * n * sizeof(double2);
}

template <int TM>
static int launch_adj(f64::AdjArgs& args, int batch, cudaStream_t st) {
  const size_t smem = (size_t)(16 * TM) * (f64::kKC + 1) * sizeof(double2) +
                      (size_t)f64::kKC * (16 * TM + 1) * sizeof(double2);
  auto kern = f64::lindblad_adjoint_f64_kernel<TM>;
  LIME_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<batch, f64::kThreads, smem, st>>>(args);
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch();
  return LIME_OK;
}

extern "C" int lime_lindblad_adjoint_f64(const LimeAdjointDesc* d, void* stream) {
  if (!d) return LIME_ERR_ARG;
  if (d->n <= 0 || d->batch <= 0 || d->seg_steps <= 0 || d->step0 < 0 || d->k_dense < 0 || d->n_obs < 0)
    return LIME_ERR_ARG;
  if (d->step0 + d->seg_steps > d->total_steps) return LIME_ERR_ARG;
  if (!d->ckpt || !d->lam || !d->heff || !d->heff_adj || !d->workspace) return LIME_ERR_ARG;
  if (!d->grad_diag || !d->grad_bond || !d->grad_gamma) return LIME_ERR_ARG;
  if (d->k_dense > 0 && (!d->l_dense || !d->l_dense_adj)) return LIME_ERR_ARG;
  if ((d->m == nullptr) != (d->m_adj == nullptr)) return LIME_ERR_ARG;
  if (d->n_obs > 0 && (!d->obs_ops || !d->obs_grad)) return LIME_ERR_ARG;
  if (d->heff_stride < 0 || d->m_stride < 0 || d->l_dense_stride < 0 || d->heff_adj_stride < 0 ||
      d->m_adj_stride < 0 || d->l_dense_adj_stride < 0 || d->obs_stride < 0)
    return LIME_ERR_ARG;
  const int pb = d->param_batch > 0 ? d->param_batch : d->batch;
  if (pb > d->batch) return LIME_ERR_ARG;
  if (d->workspace_bytes < lime_lindblad_adjoint_f64_workspace(d->n, d->batch, d->seg_steps, d->k_dense))
    return LIME_ERR_WORKSPACE;
  f64::AdjArgs a{};
  a.n = d->n; a.param_batch = pb; a.seg_steps = d->seg_steps; a.step0 = d->step0;
  a.total_steps = d->total_steps; a.k_dense = d->k_dense; a.n_obs = d->n_obs; a.obs_diag = d->obs_diag;
  a.obs_every = d->obs_every > 0 ? d->obs_every : 1;
  a.obs_per_inst = d->total_steps / a.obs_every;
  a.dt = d->dt;
  a.ckpt = reinterpret_cast<const double2*>(d->ckpt);
  a.lam = reinterpret_cast<double2*>(d->lam);
  a.heff = reinterpret_cast<const double2*>(d->heff); a.heff_stride = d->heff_stride;
  a.m = reinterpret_cast<const double2*>(d->m); a.m_stride = d->m_stride;
  a.ld = reinterpret_cast<const double2*>(d->l_dense); a.ld_stride = d->l_dense_stride;
  a.heff_adj = reinterpret_cast<const double2*>(d->heff_adj); a.heff_adj_stride = d->heff_adj_stride;
  a.m_adj = reinterpret_cast<const double2*>(d->m_adj); a.m_adj_stride = d->m_adj_stride;
  a.ld_adj = reinterpret_cast<const double2*>(d->l_dense_adj); a.ld_adj_stride = d->l_dense_adj_stride;
  a.obs_ops = reinterpret_cast<const double2*>(d->obs_ops); a.obs_stride = d->obs_stride;
  a.obs_grad = reinterpret_cast<const double2*>(d->obs_grad);
  a.g_diag = d->grad_diag; a.g_bond = d->grad_bond; a.g_gamma = d->grad_gamma;
  a.ws = reinterpret_cast<double2*>(d->workspace);
  cudaStream_t st = (cudaStream_t)stream;
  if (d->n <= 16) return launch_adj<1>(a, d->batch, st);
  if (d->n <= 32) return launch_adj<2>(a, d->batch, st);
  return launch_adj<4>(a, d->batch, st);
}
