// Batched split-precision Lindblad RK4 on the sm_103a tensor cores (tcgen05).
//
// Each CTA propagates whole density matrices (dimension n <= 64, zero-padded
// to 64) through the full time loop, one instance at a time; two CTAs share
// an SM so one's tensor-core work overlaps the other's epilogue.
//
// Per RK4 stage the generator needs X = Heff rho_s (complex 64x64x64).  It is
// one real GEMM of the block form
//     [Xr; Xi] (128 x 64) = [[Hr, -Hi], [Hi, Hr]] (128 x 128) . [rr; ri] (128 x 64)
// issued as tcgen05.mma M=128, N=64, K=16 (kind::f16, fp32 accumulation) with
// A (the Heff block, constant per instance) in tensor memory and B (the stage
// input rho_s) in shared memory (K-major, no swizzle).
//
// Accuracy.  A tcgen05.mma sums its 16 products and the accumulator exactly
// and rounds the result toward zero to fp32 (measured on GB300): every
// instruction shrinks |D| by half an ulp on average, a bias that acts like a
// slightly smaller Hamiltonian and grows into a phase error linear in time.
// The dominant product is therefore made exact:
//   A = A0 + A1 + A2:  A0 = per-row fixed point, |A0| <= 127 q_A(row);
//                      A1, A2 = fp16 of the successive residuals (~30 bits)
//   B = B0 + B1:       B0 = per-row fixed point, |B0| <= 1023 q_B(row);
//                      B1 = fp16 of the residual (~21 bits)
// with power-of-two quanta.  Every partial sum of A0.B0 over K = 128 is an
// integer multiple of q_A q_B below 2^24 (127 * 1023 * 128 < 2^24), so its
// accumulation is exact and truncation never fires.  The small products
// A1.B0 + A0.B1 + A1.B1 + A2.B0 (<= 2^-7 of X) are accumulated first through
// the same TMEM columns; their truncation bias is ~2^-27 of X.  The two
// partial results are summed in fp32 (round to nearest) by the epilogue.
//
// Epilogue (4 warps; thread t owns TMEM lane t, i.e. row t of [Xr; Xi]):
// threads 0..63 form Im f[i][:] = Xr[j][i] - Xr[i][j], threads 64..127 form
// Re f[i][:] = Xi[i][j] + Xi[j][i] (the X^dag half comes through a shared
// transpose buffer), add the dephasing jump term m_i rho_ii, and fuse the RK4
// stage combination (lime/phys.py:636-649).  The state rho is held in fp32
// registers with an fp32 compensation term in shared memory (two-sum), and
// dt/6 is carried as a float pair, so neither rounding nor the step size
// drifts over thousands of steps.  rho stays exactly Hermitian, which lets
// each thread write its own row segment of the next B operand
// (B^T row i = [Re rho[i][:], -Im rho[i][:]]).  Observables, the trace check
// and the final state are produced in FP64 from hi + lo.

#include "common.cuh"
#include "tc_ptx.cuh"

namespace lime {
namespace split {

constexpr int kN = 64;
constexpr int kThreads = 128;
constexpr int kXtStride = 68;            // floats per transpose-buffer row (conflict-free float4 rows)
constexpr uint32_t kTmemCols = 256;      // A0 [0,64) | A1 [64,128) | A2 [128,192) | D [192,256)
constexpr uint32_t kColA0 = 0, kColA1 = 64, kColA2 = 128, kColD = 192;
constexpr uint32_t kLBO = 128;           // B operand: K-direction core-matrix stride (bytes)
constexpr uint32_t kSBO = 2048;          // B operand: N-direction 8-row-group stride (bytes)
constexpr uint32_t kBopBytes = 16384;    // 64 (N) x 128 (K) fp16
constexpr float kB0Max = 1023.f;         // |B0| / q_B
constexpr double kA0Max = 127.0;         // |A0| / q_A
constexpr float kRowFloor = 8.f;         // smallest row bound used for q_B (scaled units)

struct __align__(1024) Smem {
  uint8_t bop[2][kBopBytes];             // B0 (fixed point), B1 (residual)
  float xt[128 * kXtStride];             // D transpose buffer
  float rlo[kN * kThreads];              // compensation of rho, [j][t]
  float smax[2][kThreads];               // per-thread max |B| of the last written stage input
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

__device__ __forceinline__ uint32_t pack_half2(__half lo, __half hi) {
  return (uint32_t)__half_as_ushort(lo) | ((uint32_t)__half_as_ushort(hi) << 16);
}

// x = a0 + a1 + a2: a0 on the q grid (|a0| <= 127 q), a1/a2 fp16 residuals.
__device__ __forceinline__ void split_a(double x, double q, double inv_q, __half& a0, __half& a1, __half& a2) {
  const double k = fmin(fmax(rint(x * inv_q), -kA0Max), kA0Max);
  const double v0 = k * q;
  a0 = __double2half(v0);
  const double r1 = x - v0;
  a1 = __double2half(r1);
  a2 = __double2half(r1 - (double)__half2float(a1));
}

// x = b0 + b1: b0 on the q grid (|b0| <= 1023 q), b1 = fp16(x - b0).
__device__ __forceinline__ void split_b(float x, float q, float inv_q, __half& b0, __half& b1) {
  const float k = fminf(fmaxf(rintf(x * inv_q), -kB0Max), kB0Max);
  const float v0 = k * q;
  b0 = __float2half_rn(v0);
  b1 = __float2half_rn(x - v0);
}

// Power-of-two quantum for a row whose magnitude bound is m (scaled units):
// |x| <= 1.5 m fits 1023 q with q = 2^(floor(log2(1.5 m)) - 9).
__device__ __forceinline__ void row_quantum(float m, float& q, float& inv_q) {
  const float mm = fmaxf(1.5f * m, kRowFloor);
  const int e = ilogbf(mm);
  q = ldexpf(1.f, e - 9);
  inv_q = ldexpf(1.f, 9 - e);
}

// Write 8 consecutive B^T values (chunk c of this thread's row segment).
__device__ __forceinline__ void store_b8(Smem& S, uint32_t off, const float* x, float q, float inv_q, float& mx) {
  uint32_t h0[4], h1[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    __half a0, a1, b0, b1;
    split_b(x[2 * e], q, inv_q, a0, a1);
    split_b(x[2 * e + 1], q, inv_q, b0, b1);
    h0[e] = pack_half2(a0, b0);
    h1[e] = pack_half2(a1, b1);
    mx = fmaxf(mx, fmaxf(fabsf(x[2 * e]), fabsf(x[2 * e + 1])));
  }
  *reinterpret_cast<uint4*>(S.bop[0] + off) = make_uint4(h0[0], h0[1], h0[2], h0[3]);
  *reinterpret_cast<uint4*>(S.bop[1] + off) = make_uint4(h1[0], h1[1], h1[2], h1[3]);
}

// Issue one MMA pass on thread 0 and wait for it; returns false on timeout.
template <bool kExact>
__device__ __forceinline__ bool mma_pass(uint32_t tbase, uint32_t b0_addr, uint32_t b1_addr, uint64_t* mbar,
                                         uint32_t parity, uint32_t max_wait) {
  constexpr uint32_t idesc = tc::idesc_f16(128, 64, 0);
  tc::tc_fence_after();
#pragma unroll
  for (int ks = 0; ks < 8; ++ks) {
    const uint64_t d0 = tc::smem_desc_noswizzle(b0_addr + ks * 2 * kLBO, kLBO, kSBO);
    const uint32_t acc = ks > 0 ? 1u : 0u;
    if (kExact) {
      tc::mma_f16_ts(tbase + kColD, tbase + kColA0 + ks * 8, d0, idesc, acc);
    } else {
      const uint64_t d1 = tc::smem_desc_noswizzle(b1_addr + ks * 2 * kLBO, kLBO, kSBO);
      tc::mma_f16_ts(tbase + kColD, tbase + kColA1 + ks * 8, d0, idesc, acc);
      tc::mma_f16_ts(tbase + kColD, tbase + kColA0 + ks * 8, d1, idesc, 1u);
      tc::mma_f16_ts(tbase + kColD, tbase + kColA1 + ks * 8, d1, idesc, 1u);
      tc::mma_f16_ts(tbase + kColD, tbase + kColA2 + ks * 8, d0, idesc, 1u);
    }
  }
  tc::mma_commit(mbar);
  return tc::mbar_wait_bounded(mbar, parity, max_wait);
}

__global__ void __launch_bounds__(kThreads, 2) lindblad_rk4_split_kernel(Args a) {
  extern __shared__ uint8_t smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int t = threadIdx.x, warp = t >> 5;
  const bool is_re = t >= 64;   // rows 64..127 of D hold Xi and give Re f
  const int i = t & 63;
  const int partner = is_re ? i : 64 + i;   // the other component of row i
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
  const uint32_t b0_addr = tc::smem_u32(S.bop[0]);
  const uint32_t b1_addr = tc::smem_u32(S.bop[1]);
  const uint32_t brow = (uint32_t)(i >> 3) * kSBO + (uint32_t)(i & 7) * 16u;
  const uint32_t bchunk0 = is_re ? 0u : 8u;
  const float bsign = is_re ? a.sb : -a.sb;
  uint32_t phase = 0;
  int flags = 0;
  bool aborted = false;
  int g = 0;   // stage counter (parity selects the smax buffer)

  for (int b = blockIdx.x; b < a.batch && !aborted; b += gridDim.x) {
    const int p = b % a.param_batch;
    const double2* heff = a.heff + p * a.heff_stride;
    const float mi = (a.m_diag && i < n) ? (float)a.m_diag[p * a.m_stride + i] : 0.f;

    // ---- A operand: scaled Heff block row t -> TMEM as A0 + A1 + A2 ----
    {
      double rmax = 0.0;
      for (int k = 0; k < 128; ++k) rmax = fmax(rmax, fabs(a_elem(heff, n, i, k, is_re) * a.sa_d));
      double q = 1.0, inv_q = 0.0;   // inv_q = 0: no fixed-point part for negligible rows
      if (rmax >= 0x1p-18) {
        const int e = ilogb(rmax);
        q = ldexp(1.0, e - 6);
        inv_q = ldexp(1.0, 6 - e);
      }
#pragma unroll 1
      for (int qq = 0; qq < 4; ++qq) {
        uint32_t p0[16], p1[16], p2[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          const int k = qq * 32 + 2 * c;
          __half x0, x1, x2, y0, y1, y2;
          split_a(a_elem(heff, n, i, k, is_re) * a.sa_d, q, inv_q, x0, x1, x2);
          split_a(a_elem(heff, n, i, k + 1, is_re) * a.sa_d, q, inv_q, y0, y1, y2);
          p0[c] = pack_half2(x0, y0);
          p1[c] = pack_half2(x1, y1);
          p2[c] = pack_half2(x2, y2);
        }
        tc::tmem_st16(lane_addr + kColA0 + qq * 16, p0);
        tc::tmem_st16(lane_addr + kColA1 + qq * 16, p1);
        tc::tmem_st16(lane_addr + kColA2 + qq * 16, p2);
      }
      tc::tmem_wait_st();
    }

    // ---- state: this thread's component of row i ----
    float rho[kN], acc[kN];
    const double2* r0 = a.rho + (int64_t)b * n * n;
    double dtr = 0.0;
    float mx = 0.f;
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
      mx = fmaxf(mx, fabsf(h * a.sb));
      if (is_re && j == i) dtr = v;
    }
    S.smax[g & 1][t] = mx;
    const double tr0 = block_sum2(dtr, S.red[0], t);   // (its barriers publish smax)
    float rs_diag = 0.f;   // Re rho_s[i][i] of the current stage input (RE threads)
#pragma unroll
    for (int j = 0; j < kN; ++j)
      if (j == i) rs_diag = rho[j];
    {
      float q, inv_q;
      row_quantum(fmaxf(S.smax[g & 1][t], S.smax[g & 1][partner]), q, inv_q);
      float dummy = 0.f;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = rho[8 * c + e] * bsign;
        store_b8(S, brow + (bchunk0 + c) * kLBO, x, q, inv_q, dummy);
      }
    }

#pragma unroll 1
    for (int step = 0; step < a.n_steps; ++step) {
#pragma unroll 1
      for (int s = 0; s < 4; ++s, ++g) {
        // ---- pass 1: small products into D ----
        tc::fence_proxy_async_smem();
        tc::tc_fence_before();
        __syncthreads();
        int timed_out = 0;
        if (t == 0) timed_out = mma_pass<false>(tbase, b0_addr, b1_addr, &S.mbar, phase, a.max_wait) ? 0 : 1;
        phase ^= 1u;
        if (__syncthreads_or(timed_out)) {
          aborted = true;
          break;
        }
        tc::tc_fence_after();
        float* xrow = S.xt + t * kXtStride;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float v[16];
          tc::tmem_ld16(lane_addr + kColD + q * 16, v);
#pragma unroll
          for (int e = 0; e < 4; ++e)
            *reinterpret_cast<float4*>(xrow + q * 16 + 4 * e) =
                make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
        }
        // ---- pass 2: the exact product A0.B0 into D ----
        tc::tc_fence_before();
        __syncthreads();
        if (t == 0) timed_out = mma_pass<true>(tbase, b0_addr, b1_addr, &S.mbar, phase, a.max_wait) ? 0 : 1;
        phase ^= 1u;
        if (__syncthreads_or(timed_out)) {
          aborted = true;
          break;
        }
        tc::tc_fence_after();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float v[16];
          tc::tmem_ld16(lane_addr + kColD + q * 16, v);
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            float4* p4 = reinterpret_cast<float4*>(xrow + q * 16 + 4 * e);
            const float4 o = *p4;
            *p4 = make_float4(__fadd_rn(v[4 * e], o.x), __fadd_rn(v[4 * e + 1], o.y),
                              __fadd_rn(v[4 * e + 2], o.z), __fadd_rn(v[4 * e + 3], o.w));
          }
        }
        // the quantum for the next B operand (from this stage input's row bound)
        float qb, inv_qb;
        row_quantum(fmaxf(S.smax[g & 1][t], S.smax[g & 1][partner]), qb, inv_qb);
        __syncthreads();

        const float* xcol = S.xt + (is_re ? 64 : 0) * kXtStride + i;   // X[j][i] at xcol[j * stride]
        const float cst = (s == 2) ? a.c_full : a.c_half;
        const float w = (s == 0 || s == 3) ? 1.f : 2.f;
        float rs_diag_next = rs_diag;
        float nmx = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float own[16];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float4 o = *reinterpret_cast<const float4*>(xrow + q * 16 + 4 * e);
            own[4 * e] = o.x; own[4 * e + 1] = o.y; own[4 * e + 2] = o.z; own[4 * e + 3] = o.w;
          }
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
              // fp32 dt/6 rescales time by up to 2^-24
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
            float x[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) x[e] = nxt[8 * h8 + e] * bsign;
            store_b8(S, brow + (bchunk0 + 2 * q + h8) * kLBO, x, qb, inv_qb, nmx);
          }
        }
        S.smax[(g + 1) & 1][t] = nmx;
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
    __syncthreads();   // smax / rlo of this instance are no longer read
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
