// Batched split-precision Lindblad RK4 on the sm_103a tensor cores (tcgen05).
//
// Each CTA propagates whole density matrices (dimension n <= 64, zero-padded
// to 64) through the full time loop, one instance at a time; two CTAs share
// an SM so one's tensor-core work overlaps the other's epilogue.
//
// Per RK4 stage the generator needs X = Heff rho_s (complex 64x64x64).  It is
// one real GEMM of the block form
//     [Xr; Xi] (128 x 64) = [[Hr, -Hi], [Hi, Hr]] (128 x 128) . [rr; ri] (128 x 64)
// issued as tcgen05.mma M=128, N=64, K=16 (kind::f16, fp32 accumulation):
//   * A = Heff block, power-of-two pre-scaled and split in FP64 into three
//     fp16 pieces hi + mid + lo, written once per instance into tensor
//     memory (A-from-TMEM form);
//   * B = rho_s block, pre-scaled and split into fp16 hi + lo, rewritten in
//     shared memory (K-major, no swizzle) by the epilogue of the previous
//     stage;
//   * D += Ahi.Bhi + Ahi.Blo + Amid.Bhi + Alo.Bhi into one fp32 TMEM
//     accumulator.
// With 11-bit fp16 significands the rho split carries ~22 bits (the accuracy
// of 3xTF32 at the fp16 tensor rate; a bf16 split, 8+8 bits, does not reach
// 1e-6 over thousands of steps).  Its error changes every step and averages
// out; Heff's does not (it is a fixed perturbation of the generator, whose
// phase error grows linearly in time), hence the third A piece.
//
// Epilogue (4 warps; thread t owns TMEM lane t, i.e. row t of [Xr; Xi]):
// threads 0..63 form Im f[i][:] = Xr[j][i] - Xr[i][j], threads 64..127 form
// Re f[i][:] = Xi[i][j] + Xi[j][i] (the X^dag half comes through a shared
// transpose buffer), add the dephasing jump term m_i rho_ii, and fuse the RK4
// stage combination (lime/phys.py:636-649).  The state rho is held in fp32
// registers with an fp32 compensation term in shared memory (two-sum), so
// rounding does not accumulate over thousands of steps.  rho stays exactly
// Hermitian, which lets each thread write its own row segment of the next B
// operand (B^T row i = [Re rho[i][:], -Im rho[i][:]]).  Observables, the
// trace check and the final state are produced in FP64 from hi + lo.

#include "common.cuh"
#include "tc_ptx.cuh"

namespace lime {
namespace split {

constexpr int kN = 64;
constexpr int kThreads = 128;
constexpr int kXtStride = 68;            // floats per transpose-buffer row (conflict-free float4 rows)
constexpr uint32_t kTmemCols = 256;      // A hi [0,64) | A mid [64,128) | A lo [128,192) | D [192,256)
constexpr uint32_t kColAhi = 0, kColAmid = 64, kColAlo = 128, kColD = 192;
constexpr uint32_t kLBO = 128;           // B operand: K-direction core-matrix stride (bytes)
constexpr uint32_t kSBO = 2048;          // B operand: N-direction 8-row-group stride (bytes)
constexpr uint32_t kBopBytes = 16384;    // 64 (N) x 128 (K) fp16

struct __align__(1024) Smem {
  uint8_t bop[2][kBopBytes];             // B operand hi, lo
  float xt[128 * kXtStride];             // D transpose buffer
  float rlo[kN * kThreads];              // compensation of rho, [j][t]
  double red[2][kThreads / 32];
  uint64_t mbar;
  uint32_t tmem_base;
};

struct Args {
  int n, batch, param_batch, n_steps, step0, obs_mode, n_obs, obs_every, obs_per_inst;
  float sb, inv_sab, c_half, c_full, c_sixth, c_sixth_lo;
  double sa_d;
  double trace_tol;
  double2* rho;
  const double2* heff; int64_t heff_stride;
  const double* m_diag; int64_t m_stride;
  const double2* obs_ops; int64_t obs_stride;
  double2* obs_out;
  int32_t* status;
  uint32_t max_wait;
};

__device__ __forceinline__ double block_sum2(double v, double* red, int t) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((t & 31) == 0) red[t >> 5] = v;
  __syncthreads();
  return red[0] + red[1] + red[2] + red[3];
}

// A row t of the block matrix, in FP64 (pre-scaling applied by the caller).
__device__ __forceinline__ double a_elem(const double2* heff, int n, int i, int k, bool xi_row) {
  const int kk = k & 63;
  if (i >= n || kk >= n) return 0.0;
  const double2 h = heff[(int64_t)i * n + kk];
  if (!xi_row) return k < 64 ? h.x : -h.y;   // Xr rows: [Hr, -Hi]
  return k < 64 ? h.y : h.x;                 // Xi rows: [Hi,  Hr]
}

// Three-way fp16 split of an FP64 pair: x = h1 + h2 + h3 to ~33 bits.
__device__ __forceinline__ void split3_f16(double x0, double x1, uint32_t& p1, uint32_t& p2, uint32_t& p3) {
  __half a1 = __double2half(x0), b1 = __double2half(x1);
  const double r0 = x0 - (double)__half2float(a1), s0 = x1 - (double)__half2float(b1);
  __half a2 = __double2half(r0), b2 = __double2half(s0);
  const double r1 = r0 - (double)__half2float(a2), s1 = s0 - (double)__half2float(b2);
  __half a3 = __double2half(r1), b3 = __double2half(s1);
  p1 = (uint32_t)__half_as_ushort(a1) | ((uint32_t)__half_as_ushort(b1) << 16);
  p2 = (uint32_t)__half_as_ushort(a2) | ((uint32_t)__half_as_ushort(b2) << 16);
  p3 = (uint32_t)__half_as_ushort(a3) | ((uint32_t)__half_as_ushort(b3) << 16);
}

__global__ void __launch_bounds__(kThreads, 2) lindblad_rk4_split_kernel(Args a) {
  extern __shared__ uint8_t smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int t = threadIdx.x, warp = t >> 5;
  const bool is_re = t >= 64;   // rows 64..127 of D hold Xi and give Re f
  const int i = t & 63;
  const int n = a.n;

  if (warp == 0) {
    tc::tmem_alloc(&S.tmem_base, kTmemCols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(&S.mbar, 1);
    tc::mbar_fence_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = S.tmem_base;
  const uint32_t lane_addr = tbase + ((uint32_t)(warp * 32) << 16);
  constexpr uint32_t idesc = tc::idesc_f16(128, 64, 0);
  const uint32_t bop_hi = tc::smem_u32(S.bop[0]);
  const uint32_t bop_lo = tc::smem_u32(S.bop[1]);
  const uint32_t brow = (uint32_t)(i >> 3) * kSBO + (uint32_t)(i & 7) * 16u;
  const uint32_t bchunk0 = is_re ? 0u : 8u;
  const float bsign = is_re ? a.sb : -a.sb;
  uint32_t phase = 0;
  int flags = 0;
  bool aborted = false;

  for (int b = blockIdx.x; b < a.batch && !aborted; b += gridDim.x) {
    const int p = b % a.param_batch;
    const double2* heff = a.heff + p * a.heff_stride;
    const float mi = (a.m_diag && i < n) ? (float)a.m_diag[p * a.m_stride + i] : 0.f;

    // ---- A operand: scaled Heff block -> TMEM (lane t = row t), 3 fp16 pieces ----
    // Heff is the same for every step, so its representation error is a
    // fixed perturbation of the generator whose phase error grows linearly
    // in time; the third piece pushes it to ~2^-33.
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
      uint32_t hi[16], mid[16], lo[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int k = q * 32 + 2 * c;
        split3_f16(a_elem(heff, n, i, k, is_re) * a.sa_d, a_elem(heff, n, i, k + 1, is_re) * a.sa_d,
                   hi[c], mid[c], lo[c]);
      }
      tc::tmem_st16(lane_addr + kColAhi + q * 16, hi);
      tc::tmem_st16(lane_addr + kColAmid + q * 16, mid);
      tc::tmem_st16(lane_addr + kColAlo + q * 16, lo);
    }
    tc::tmem_wait_st();

    // ---- state: this thread's component of row i ----
    float rho[kN], acc[kN];
    const double2* r0 = a.rho + (int64_t)b * n * n;
    double dtr = 0.0;
#pragma unroll
    for (int j = 0; j < kN; ++j) {
      double v = 0.0;
      if (i < n && j < n) {
        const double2 z = r0[(int64_t)i * n + j];
        v = is_re ? z.x : z.y;
      }
      const float h = (float)v;
      rho[j] = h;
      S.rlo[j * kThreads + t] = (float)(v - (double)h);
      if (is_re && j == i) dtr = v;
    }
    const double tr0 = block_sum2(dtr, S.red[0], t);
    float rs_diag = 0.f;   // Re rho_s[i][i] of the current stage input (RE threads)
#pragma unroll
    for (int j = 0; j < kN; ++j)
      if (j == i) rs_diag = rho[j];
    // stage-0 B operand
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      uint32_t h[4], l[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) tc::split2_f16(rho[8 * c + 2 * e] * bsign, rho[8 * c + 2 * e + 1] * bsign, h[e], l[e]);
      const uint32_t off = brow + (bchunk0 + c) * kLBO;
      *reinterpret_cast<uint4*>(S.bop[0] + off) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4*>(S.bop[1] + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }

#pragma unroll 1
    for (int step = 0; step < a.n_steps; ++step) {
#pragma unroll 1
      for (int s = 0; s < 4; ++s) {
        // B operand (generic-proxy writes) -> visible to the tensor core
        tc::fence_proxy_async_smem();
        tc::tc_fence_before();
        __syncthreads();
        int timed_out = 0;
        if (t == 0) {
          tc::tc_fence_after();
#pragma unroll
          for (int ks = 0; ks < 8; ++ks) {
            const uint64_t dh = tc::smem_desc_noswizzle(bop_hi + ks * 2 * kLBO, kLBO, kSBO);
            const uint64_t dl = tc::smem_desc_noswizzle(bop_lo + ks * 2 * kLBO, kLBO, kSBO);
            tc::mma_f16_ts(tbase + kColD, tbase + kColAhi + ks * 8, dh, idesc, ks > 0 ? 1u : 0u);
            tc::mma_f16_ts(tbase + kColD, tbase + kColAhi + ks * 8, dl, idesc, 1u);
            tc::mma_f16_ts(tbase + kColD, tbase + kColAmid + ks * 8, dh, idesc, 1u);
            tc::mma_f16_ts(tbase + kColD, tbase + kColAlo + ks * 8, dh, idesc, 1u);
          }
          tc::mma_commit(&S.mbar);
          timed_out = tc::mbar_wait_bounded(&S.mbar, phase, a.max_wait) ? 0 : 1;
        }
        phase ^= 1u;
        if (__syncthreads_or(timed_out)) {
          aborted = true;
          break;
        }
        tc::tc_fence_after();

        // D row t -> transpose buffer
        float* xrow = S.xt + t * kXtStride;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float v[16];
          tc::tmem_ld16(lane_addr + kColD + q * 16, v);
#pragma unroll
          for (int e = 0; e < 4; ++e)
            *reinterpret_cast<float4*>(xrow + q * 16 + 4 * e) = make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
        }
        __syncthreads();

        const float* xcol = S.xt + (is_re ? 64 : 0) * kXtStride + i;   // X[j][i] at xcol[j * stride]
        const float cst = (s == 2) ? a.c_full : a.c_half;
        const float w = (s == 0 || s == 3) ? 1.f : 2.f;
        float rs_diag_next = rs_diag;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float own[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) own[e] = xrow[q * 16 + e];
          float nxt[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int j = q * 16 + e;
            const float tr = xcol[j * kXtStride];
            float f = (is_re ? (own[e] + tr) : (tr - own[e])) * a.inv_sab;
            if (is_re && j == i) f = __fmaf_rn(mi, rs_diag, f);
            if (s == 0) {
              acc[j] = f;
            } else if (s < 3) {
              acc[j] = __fmaf_rn(w, f, acc[j]);
            }
            if (s < 3) {
              nxt[e] = __fmaf_rn(cst, f, rho[j]);
            } else {
              // increment (k1 + 2k2 + 2k3 + k4) dt/6 with dt/6 carried as a
              // float pair and the product's rounding residual kept: a plain
              // fp32 dt/6 rescales time by up to 2^-24, a phase error that
              // grows linearly in time
              const float ksum = __fadd_rn(acc[j], f);
              const float inc = __fmul_rn(ksum, a.c_sixth);
              const float inc_res = __fmaf_rn(ksum, a.c_sixth, -inc);
              const float inc_lo = __fmaf_rn(ksum, a.c_sixth_lo, inc_res);
              // two-sum of rho_hi + inc, errors folded into the compensation term
              const float x = rho[j];
              const float sum = __fadd_rn(x, inc);
              const float bv = __fsub_rn(sum, x);
              const float err = __fadd_rn(__fsub_rn(x, __fsub_rn(sum, bv)), __fsub_rn(inc, bv));
              float lo = __fadd_rn(S.rlo[j * kThreads + t], __fadd_rn(err, inc_lo));
              const float hi2 = __fadd_rn(sum, lo);
              lo = __fsub_rn(lo, __fsub_rn(hi2, sum));
              rho[j] = hi2;
              S.rlo[j * kThreads + t] = lo;
              nxt[e] = hi2;
            }
            if (j == i) rs_diag_next = nxt[e];
          }
          // next B operand: two 8-wide chunks
#pragma unroll
          for (int h8 = 0; h8 < 2; ++h8) {
            uint32_t hh[4], ll[4];
#pragma unroll
            for (int e = 0; e < 4; ++e)
              tc::split2_f16(nxt[8 * h8 + 2 * e] * bsign, nxt[8 * h8 + 2 * e + 1] * bsign, hh[e], ll[e]);
            const uint32_t off = brow + (bchunk0 + 2 * q + h8) * kLBO;
            *reinterpret_cast<uint4*>(S.bop[0] + off) = make_uint4(hh[0], hh[1], hh[2], hh[3]);
            *reinterpret_cast<uint4*>(S.bop[1] + off) = make_uint4(ll[0], ll[1], ll[2], ll[3]);
          }
        }
        rs_diag = rs_diag_next;
      }
      if (aborted) break;

      // ---- observables / trace after the step ----
      const int gstep = a.step0 + step;
      if (((gstep + 1) % a.obs_every) == 0) {
        const int slot = (gstep + 1) / a.obs_every - 1;
        double2* orow = a.obs_out + ((int64_t)b * a.obs_per_inst + slot) * a.n_obs;
        if (a.obs_mode == 1) {
          if (is_re && i < a.n_obs)
            orow[i] = make_double2((double)rs_diag + (double)S.rlo[i * kThreads + t], 0.0);
        } else if (a.obs_mode == 2) {
          const double2* E0 = a.obs_ops + p * a.obs_stride;
          for (int o = 0; o < a.n_obs; ++o) {
            const double2* E = E0 + (int64_t)o * n * n;
            float pr = 0.f, pi = 0.f;
            if (i < n) {
#pragma unroll
              for (int j = 0; j < kN; ++j) {
                if (j < n) {
                  const double2 e = E[(int64_t)j * n + i];   // E[j][i]
                  const float er = (float)e.x, ei = (float)e.y;
                  if (is_re) {
                    pr = __fmaf_rn(er, rho[j], pr);
                    pi = __fmaf_rn(ei, rho[j], pi);
                  } else {
                    pr = __fmaf_rn(-ei, rho[j], pr);
                    pi = __fmaf_rn(er, rho[j], pi);
                  }
                }
              }
            }
            const double sr = block_sum2((double)pr, S.red[0], t);
            const double si = block_sum2((double)pi, S.red[1], t);
            if (t == 0) orow[o] = make_double2(sr, si);
          }
        }
        if (a.trace_tol > 0.0) {
          const double d = (is_re && i < n) ? (double)rs_diag + (double)S.rlo[i * kThreads + t] : 0.0;
          const double tr = block_sum2(d, S.red[0], t);
          if (fabs(tr - tr0) > a.trace_tol * fmax(1.0, fabs(tr0))) flags |= LIME_FLAG_TRACE_DRIFT;
        }
      }
    }
    if (aborted) break;

    // ---- final state: rho = hi + lo in FP64 ----
    if (i < n) {
      double* out = reinterpret_cast<double*>(a.rho + (int64_t)b * n * n);
#pragma unroll
      for (int j = 0; j < kN; ++j) {
        if (j < n) {
          const double v = (double)rho[j] + (double)S.rlo[j * kThreads + t];
          if (!isfinite(v)) flags |= LIME_FLAG_NONFINITE;
          out[2 * ((int64_t)i * n + j) + (is_re ? 0 : 1)] = v;
        }
      }
    }
  }

  if (aborted) {
    flags |= LIME_FLAG_TIMEOUT;
    // let any tensor-core work still in flight drain before TMEM is released
    if (t == 0) tc::mbar_wait_bounded(&S.mbar, phase ^ 1u, a.max_wait);
  }
  if (flags) atomicOr(a.status, flags);
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tbase, kTmemCols);
  }
}

}  // namespace split
}  // namespace lime

using namespace lime;

static int g_num_sms = 0;

extern "C" int lime_lindblad_rk4_split(const LimeLindbladSplitDesc* d, void* stream) {
  if (!d) return LIME_ERR_ARG;
  if (d->n <= 0 || d->batch <= 0 || d->n_steps < 0 || d->n_obs < 0) return LIME_ERR_ARG;
  if (d->n > split::kN) return LIME_ERR_UNSUPPORTED;
  if (!d->rho || !d->heff || !d->status) return LIME_ERR_ARG;
  if (d->obs_mode < 0 || d->obs_mode > 2) return LIME_ERR_ARG;
  if (d->obs_mode == 1 && d->n_obs > d->n) return LIME_ERR_ARG;
  if (d->obs_mode != 0 && d->n_obs > 0 && !d->obs_out) return LIME_ERR_ARG;
  if (d->obs_mode == 2 && d->n_obs > 0 && !d->obs_ops) return LIME_ERR_ARG;
  if (d->heff_stride < 0 || d->m_stride < 0 || d->obs_stride < 0) return LIME_ERR_ARG;
  if (d->scale_a_log2 < -60 || d->scale_a_log2 > 60 || d->scale_b_log2 < -60 || d->scale_b_log2 > 60)
    return LIME_ERR_ARG;
  const int pb = d->param_batch > 0 ? d->param_batch : d->batch;
  if (pb > d->batch) return LIME_ERR_ARG;
  if (!(d->dt == d->dt)) return LIME_ERR_ARG;
  if (d->n_steps == 0) return LIME_OK;
  if (g_num_sms == 0) {
    int dev = 0;
    LIME_CUDA_TRY(cudaGetDevice(&dev));
    LIME_CUDA_TRY(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
  }
  split::Args a{};
  a.n = d->n; a.batch = d->batch; a.param_batch = pb;
  a.obs_mode = d->n_obs > 0 ? d->obs_mode : 0;
  a.n_obs = d->n_obs;
  a.obs_every = d->obs_every > 0 ? d->obs_every : 1;
  a.obs_per_inst = d->n_steps / a.obs_every;
  a.sa_d = ldexp(1.0, d->scale_a_log2);
  a.sb = ldexpf(1.f, d->scale_b_log2);
  a.inv_sab = ldexpf(1.f, -(d->scale_a_log2 + d->scale_b_log2));
  a.c_half = (float)(d->dt / 2.0);
  a.c_full = (float)d->dt;
  a.c_sixth = (float)(d->dt / 6.0);
  a.c_sixth_lo = (float)(d->dt / 6.0 - (double)a.c_sixth);
  a.trace_tol = d->trace_tol;
  a.rho = reinterpret_cast<double2*>(d->rho);
  a.heff = reinterpret_cast<const double2*>(d->heff); a.heff_stride = d->heff_stride;
  a.m_diag = d->m_diag; a.m_stride = d->m_stride;
  a.obs_ops = reinterpret_cast<const double2*>(d->obs_ops); a.obs_stride = d->obs_stride;
  a.obs_out = reinterpret_cast<double2*>(d->obs_out);
  a.status = d->status;
  a.max_wait = 1u << 26;
  const int ctas_per_sm = d->ctas_per_sm > 0 ? d->ctas_per_sm : 2;
  const int grid = (int)((d->batch < ctas_per_sm * g_num_sms) ? d->batch : ctas_per_sm * g_num_sms);
  const size_t smem = sizeof(split::Smem) + 1024;
  LIME_CUDA_TRY(cudaFuncSetAttribute(split::lindblad_rk4_split_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // bounded launches: about 2^22 instance-steps per launch
  const double per_cta = (double)((d->batch + grid - 1) / grid);
  int chunk = (int)fmax(1.0, fmin((double)d->n_steps, 4194304.0 / (per_cta * grid)));
  if (a.obs_every > 1) chunk = ((chunk + a.obs_every - 1) / a.obs_every) * a.obs_every;
  cudaStream_t st = (cudaStream_t)stream;
  for (int s0 = 0; s0 < d->n_steps; s0 += chunk) {
    a.step0 = s0;
    a.n_steps = (d->n_steps - s0 < chunk) ? d->n_steps - s0 : chunk;
    split::lindblad_rk4_split_kernel<<<grid, split::kThreads, smem, st>>>(a);
    LIME_CUDA_TRY(cudaGetLastError());
    count_launch();
  }
  return LIME_OK;
}
