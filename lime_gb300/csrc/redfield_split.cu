// Split-precision Bloch-Redfield RK4 on the sm_103a tensor cores (tcgen05).
//
// Per RK4 stage the generator application over the right-hand-side block is
// one large complex GEMM Y = L S (L: D x D, S: D x R).  It runs as the real
// GEMM
//     [Yr | Yi] (D x 2R) = [Lr | Li] (D x 2D) . [[Sr, Si], [-Si, Sr]] (2D x 2R)
// so the big operand L is streamed once per stage without duplication.  Both
// operands live in global memory pre-tiled in the canonical K-major,
// no-swizzle UMMA layout: every (128-row tile, 64-wide K chunk) block is one
// contiguous 16 KB piece, moved by the bulk-copy (TMA) engine with
// cp.async.bulk into a two-stage shared-memory ring and completed on
// mbarriers (two 64-K stages measured faster than four 32-K ones).
//
// Warp roles per CTA (one 128 x 128 output tile, 320 threads, 1 CTA/SM):
//   warp 0      producer: bulk copies of 5 pieces per K chunk (80 KB)
//   warp 1      MMA issuer: tcgen05.mma M=128 N=128 K=16, kind::f16
//   warps 2..9  epilogue: drain TMEM accumulators into fp32 two-sum
//               accumulators (hi words in registers, lo words in shared
//               memory), then the fused RK4 stage update
//
// Precision (the same scheme as the Lindblad split kernel): A = L pieces
// A0 (per-row 7-bit fixed point) + A1 + A2 (fp16 residuals), B = S pieces
// B0 (10-bit fixed point, one quantum for the run) + B1 (fp16 residual).  A
// tcgen05.mma rounds its fp32 result toward zero, so the dominant product
// A0.B0 is kept exact: it is accumulated over 128 K (integer multiples of
// q_A q_B below 2^24) in its own TMEM accumulator D0, the small products
// A1.B0 + A0.B1 + A1.B1 + A2.B0 in D1; every 128 K D0 enters an fp32
// two-sum (hi, lo) and D1 is added to lo, round to nearest.  TMEM: D0/D1
// double buffered, 4 x 128 = 512 columns, so the MMAs of the next 128 K
// overlap the promotion of the previous ones.
//
// RK4 state (lime/oqs.py:453-462, lime/phys.py:636-649): P = hi + lo fp32
// and the stage accumulator, component-planar [2R][D] (column jj < R is
// Re vec rho_jj, jj >= R is Im vec rho_{jj-R}); after the last MMA the
// epilogue parks the stage derivative tile in the idle copy ring and updates
// the state in 8-row runs, writing the next stage input straight into the
// other B buffer as 16-byte stores (ping-pong across stages).

#include "common.cuh"
#include "tc_ptx.cuh"

namespace lime {
namespace rsp {

constexpr int kBM = 128, kBN = 128;   // output tile
constexpr int kCK = 64;                            // K per chunk (one ring stage)
constexpr int kGroup = 128 / kCK;                  // chunks per exactly accumulated 128 K
constexpr uint32_t kPiece = 128 * kCK * 2;         // 128 x 64 fp16 = 16 KB
constexpr int kStages = 2;
constexpr int kThreads = 320;
constexpr int kEpiThreads = 256;
constexpr uint32_t kLBO = 128, kSBO = kCK * 16;    // canonical K-major block strides (bytes)
constexpr uint32_t kTmemCols = 512;
constexpr double kA0Max = 127.0;
constexpr float kBMax = 8192.f;                    // |B| bound of the 10-bit fixed point (q_B = 8)
constexpr int kFStride = kBN + 4;                  // padded row of the parked derivative tile (floats)

struct __align__(1024) Smem {
  uint8_t stage[kStages][5][kPiece];               // A0 A1 A2 B0 B1; derivative tile after the last MMA
  float lo[kBN * kBM];                             // low words of the fp32 two-sum accumulators, [col][row]
  uint64_t full[kStages], empty[kStages], accf[2], acce[2], drain;
  uint32_t tmem_base;
  int abort;
};
static_assert((size_t)kBN * kFStride * sizeof(float) <= sizeof(Smem::stage), "derivative tile fits the ring");

// byte offset of (row, k) inside one 128 x kCK block
__host__ __device__ __forceinline__ uint32_t blk_off(int row, int k) {
  return (uint32_t)(row >> 3) * kSBO + (uint32_t)(k >> 3) * kLBO + (uint32_t)(row & 7) * 16u +
         (uint32_t)(k & 7) * 2u;
}
__host__ __device__ __forceinline__ size_t piece_off(int KC, int n, int k) {
  return ((size_t)(n >> 7) * KC + k / kCK) * kPiece + blk_off(n & 127, k % kCK);
}

struct StageArgs {
  int Dp, W, KC, MT, NT, stage;      // W = 2 Rp output columns, KC = 2Dp / kCK chunks, NT = W / 128
  int KS, groups_per_split;          // observable pass: K split over KS CTAs, 128-K groups each
  float inv_sb, sb, magic_b, c_half, c_full, c_sixth, c_sixth_lo;
  const uint8_t* A[3];               // pre-tiled [MT][KC] blocks
  const float* row_inv;              // per-row inverse operand scale (powers of two; 0 on padding)
  const uint8_t* Bc[2];              // current stage input pieces, pre-tiled [NT][KC]
  uint8_t* Bn[2];                    // next stage input pieces
  float* Phi;                        // [W][Dp]
  float* Plo;
  float* Acc;
  int Rp, R, n_obs;
  double* obs;                       // observable pass: [R][n_obs] complex, accumulated
  int32_t* status;
  uint32_t max_wait;
};

// ---------------------------------------------------------------- B operand writes
__device__ __forceinline__ void split_b(float x, float magic, float& v0, float& v1) {
  v0 = __fsub_rn(__fadd_rn(x, magic), magic);
  v1 = __fsub_rn(x, v0);
}

// one element of the stage input (scaled) into both of its B^T positions:
// Re -> (j, d), (j+R, Dp+d); Im -> -Im at (j, Dp+d), +Im at (j+R, d)
__device__ __forceinline__ void scatter_b1(const StageArgs& a, int d, int jj, float x) {
  float v0, v1;
  split_b(x, a.magic_b, v0, v1);
  const __half p0 = __float2half_rn(v0), p1 = __float2half_rn(v1);
  const __half m0 = __hneg(p0), m1 = __hneg(p1);
  size_t o1, o2;
  __half s0 = p0, s1 = p1;
  if (jj < a.Rp) {
    o1 = piece_off(a.KC, jj, d);
    o2 = piece_off(a.KC, jj + a.Rp, a.Dp + d);
  } else {
    const int j = jj - a.Rp;
    o1 = piece_off(a.KC, j + a.Rp, d);
    o2 = piece_off(a.KC, j, a.Dp + d);
    s0 = m0; s1 = m1;       // the (j, Dp+d) copy is negated
  }
  *reinterpret_cast<__half*>(a.Bn[0] + o1) = p0;
  *reinterpret_cast<__half*>(a.Bn[1] + o1) = p1;
  *reinterpret_cast<__half*>(a.Bn[0] + o2) = s0;
  *reinterpret_cast<__half*>(a.Bn[1] + o2) = s1;
}

// eight consecutive rows d..d+7 (d % 8 == 0) of one column jj: two 16-byte
// stores per piece
__device__ __forceinline__ void scatter_b8(const StageArgs& a, int d, int jj, const float (&x)[8]) {
  uint32_t h0[4], h1[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float a0, a1, b0, b1;
    split_b(x[2 * i], a.magic_b, a0, a1);
    split_b(x[2 * i + 1], a.magic_b, b0, b1);
    const __half2 p = __floats2half2_rn(a0, b0);
    const __half2 q = __floats2half2_rn(a1, b1);
    h0[i] = *reinterpret_cast<const uint32_t*>(&p);
    h1[i] = *reinterpret_cast<const uint32_t*>(&q);
  }
  const uint4 P0 = make_uint4(h0[0], h0[1], h0[2], h0[3]);
  const uint4 P1 = make_uint4(h1[0], h1[1], h1[2], h1[3]);
  const uint32_t sg = 0x80008000u;
  const uint4 N0 = make_uint4(h0[0] ^ sg, h0[1] ^ sg, h0[2] ^ sg, h0[3] ^ sg);
  const uint4 N1 = make_uint4(h1[0] ^ sg, h1[1] ^ sg, h1[2] ^ sg, h1[3] ^ sg);
  size_t o1, o2;
  bool neg2 = false;
  if (jj < a.Rp) {
    o1 = piece_off(a.KC, jj, d);
    o2 = piece_off(a.KC, jj + a.Rp, a.Dp + d);
  } else {
    const int j = jj - a.Rp;
    o1 = piece_off(a.KC, j + a.Rp, d);
    o2 = piece_off(a.KC, j, a.Dp + d);
    neg2 = true;
  }
  *reinterpret_cast<uint4*>(a.Bn[0] + o1) = P0;
  *reinterpret_cast<uint4*>(a.Bn[1] + o1) = P1;
  *reinterpret_cast<uint4*>(a.Bn[0] + o2) = neg2 ? N0 : P0;
  *reinterpret_cast<uint4*>(a.Bn[1] + o2) = neg2 ? N1 : P1;
}

__device__ __forceinline__ void ld8(const float* p, float (&v)[8]) {
  const float4 x = *reinterpret_cast<const float4*>(p);
  const float4 y = *reinterpret_cast<const float4*>(p + 4);
  v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w; v[4] = y.x; v[5] = y.y; v[6] = y.z; v[7] = y.w;
}
__device__ __forceinline__ void st8(float* p, const float (&v)[8]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  *reinterpret_cast<float4*>(p + 4) = make_float4(v[4], v[5], v[6], v[7]);
}

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory"); }

// kObserve = false: one RK4 stage, Y = L S over the full K, fused stage
// update.  kObserve = true: observables <E_o> = sum_d Et[o][d] P[d][r] of
// the state held in Bc, K split over KS CTAs whose fp64 partial sums are
// added atomically into a.obs.
template <bool kObserve>
__global__ void __launch_bounds__(kThreads, 1) gemm_kernel(StageArgs a) {
  extern __shared__ uint8_t smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int tile = kObserve ? (int)(blockIdx.x % (a.MT * a.NT)) : (int)blockIdx.x;
  const int mt = tile / a.NT, nt = tile % a.NT;
  int c0 = 0, KC = a.KC;                      // this CTA's chunk range [c0, c0 + KC)
  if (kObserve) {
    const int ks = blockIdx.x / (a.MT * a.NT);
    const int g0 = ks * a.groups_per_split;
    const int g1 = min(g0 + a.groups_per_split, a.KC / kGroup);
    c0 = kGroup * g0;
    KC = kGroup * max(g1 - g0, 0);
  }
  const int KCall = a.KC;

  if (warp == 0) {
    tc::tmem_alloc(&S.tmem_base, kTmemCols);
    tc::tmem_relinquish();
  }
  if (t == 32) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&S.full[s], 1);
      tc::mbar_init(&S.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&S.accf[b], 1);
      tc::mbar_init(&S.acce[b], kEpiThreads);
    }
    tc::mbar_init(&S.drain, 1);
    S.abort = 0;
    tc::mbar_fence_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = S.tmem_base;

  if (warp == 0) {
    // ---------------- producer
    if (lane == 0) {
      int issued = 0;
      for (int c = 0; c < KC; ++c) {
        const int s = c % kStages;
        const uint32_t ph = (uint32_t)(c / kStages) & 1u;
        if (!tc::mbar_wait_bounded(&S.empty[s], ph ^ 1u, a.max_wait)) { atomicExch(&S.abort, 1); break; }
        if (*(volatile int*)&S.abort) break;
        issued = c + 1;
        tc::mbar_arrive_expect_tx(&S.full[s], 5 * kPiece);
        const size_t ao = ((size_t)mt * KCall + c0 + c) * kPiece;
        const size_t bo = ((size_t)nt * KCall + c0 + c) * kPiece;
        tc::bulk_g2s(S.stage[s][0], a.A[0] + ao, kPiece, &S.full[s]);
        tc::bulk_g2s(S.stage[s][1], a.A[1] + ao, kPiece, &S.full[s]);
        tc::bulk_g2s(S.stage[s][2], a.A[2] + ao, kPiece, &S.full[s]);
        tc::bulk_g2s(S.stage[s][3], a.Bc[0] + bo, kPiece, &S.full[s]);
        tc::bulk_g2s(S.stage[s][4], a.Bc[1] + bo, kPiece, &S.full[s]);
      }
      // the copies of the last (up to kStages) issued chunks have landed before exit
      for (int c = issued - 1; c >= 0 && c >= issued - kStages; --c)
        tc::mbar_wait_bounded(&S.full[c % kStages], (uint32_t)(c / kStages) & 1u, a.max_wait);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_f16(kBM, kBN, 0);
      for (int c = 0; c < KC; ++c) {
        const int s = c % kStages;
        const uint32_t ph = (uint32_t)(c / kStages) & 1u;
        const int p = c / kGroup, b = p & 1;
        const bool first = (c % kGroup) == 0;
        const bool last = (c % kGroup) == kGroup - 1;
        if (!tc::mbar_wait_bounded(&S.full[s], ph, a.max_wait)) { atomicExch(&S.abort, 1); break; }
        if (first && !tc::mbar_wait_bounded(&S.acce[b], ((uint32_t)(p >> 1) & 1u) ^ 1u, a.max_wait)) {
          atomicExch(&S.abort, 1);
          break;
        }
        if (*(volatile int*)&S.abort) break;
        tc::tc_fence_after();
        const uint32_t d0 = tbase + (uint32_t)(2 * b) * 128u;
        const uint32_t d1 = d0 + 128u;
        const uint32_t base = tc::smem_u32(S.stage[s][0]);
#pragma unroll
        for (int ks = 0; ks < kCK / 16; ++ks) {
          const uint32_t ko = (uint32_t)ks * 2u * kLBO;
          const uint64_t a0 = tc::smem_desc_noswizzle(base + 0 * kPiece + ko, kLBO, kSBO);
          const uint64_t a1 = tc::smem_desc_noswizzle(base + 1 * kPiece + ko, kLBO, kSBO);
          const uint64_t a2 = tc::smem_desc_noswizzle(base + 2 * kPiece + ko, kLBO, kSBO);
          const uint64_t b0 = tc::smem_desc_noswizzle(base + 3 * kPiece + ko, kLBO, kSBO);
          const uint64_t b1 = tc::smem_desc_noswizzle(base + 4 * kPiece + ko, kLBO, kSBO);
          const uint32_t acc = (first && ks == 0) ? 0u : 1u;
          tc::mma_f16_ss(d0, a0, b0, idesc, acc);
          tc::mma_f16_ss(d1, a1, b0, idesc, acc);
          tc::mma_f16_ss(d1, a0, b1, idesc, 1u);
          tc::mma_f16_ss(d1, a1, b1, idesc, 1u);
          tc::mma_f16_ss(d1, a2, b0, idesc, 1u);
        }
        tc::mma_commit(&S.empty[s]);
        if (last) tc::mma_commit(&S.accf[b]);
      }
      // every MMA this thread issued has completed before TMEM is released
      tc::mma_commit(&S.drain);
      tc::mbar_wait_bounded(&S.drain, 0u, a.max_wait);
    }
  } else {
    // ---------------- epilogue: 8 warps, TMEM lane quadrant warp & 3, column half
    const int lq = warp & 3;
    const int h = (warp - 2) >> 2;
    const int r = lq * 32 + lane;
    const uint32_t lane_addr = tbase + ((uint32_t)(lq * 32) << 16);
    // hi words in registers, lo words in shared memory (each thread owns its
    // 64 entries; lanes hit consecutive words)
    float hi[64];
    float* lo = S.lo + (64 * h) * kBM + r;
#pragma unroll
    for (int c = 0; c < 64; ++c) { hi[c] = 0.f; lo[c * kBM] = 0.f; }
    const int n_pairs = KC / kGroup;
    bool ok = true;
    for (int p = 0; p < n_pairs; ++p) {
      const int b = p & 1;
      if (!tc::mbar_wait_bounded(&S.accf[b], (uint32_t)(p >> 1) & 1u, a.max_wait)) {
        atomicExch(&S.abort, 1);
        ok = false;
        break;
      }
      tc::tc_fence_after();
      const uint32_t d0 = lane_addr + (uint32_t)(2 * b) * 128u + 64u * h;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        // (one load and wait per accumulator measured faster than both loads
        // under one wait)
        float v[16], er[16];
        tc::tmem_ld16(d0 + 16 * q, v);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          // exact D0 into the two-sum
          const float x = v[e];
          const float sm = __fadd_rn(hi[16 * q + e], x);
          const float bv = __fsub_rn(sm, hi[16 * q + e]);
          er[e] = __fadd_rn(__fsub_rn(hi[16 * q + e], __fsub_rn(sm, bv)), __fsub_rn(x, bv));
          hi[16 * q + e] = sm;
        }
        tc::tmem_ld16(d0 + 128u + 16 * q, v);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          float* l = lo + (16 * q + e) * kBM;
          *l = __fadd_rn(*l, __fadd_rn(er[e], v[e]));
        }
      }
      tc::tc_fence_before();
      tc::mbar_arrive(&S.acce[b]);
    }
    // park the derivative tile in the ring: every MMA has completed once the
    // last accumulator pair was seen, so the tensor core reads no operand
    const float rs = __fmul_rn(a.row_inv[mt * kBM + r], a.inv_sb);
    if (kObserve) {
      const int o = mt * kBM + r;
      if (ok && o < a.n_obs && KC > 0) {
        const double rsd = (double)rs;
#pragma unroll
        for (int c = 0; c < 64; ++c) {
          const int jj = nt * kBN + 64 * h + c;
          const int j = jj < a.Rp ? jj : jj - a.Rp;
          if (j < a.R) {
            const double f = ((double)hi[c] + (double)lo[c * kBM]) * rsd;
            atomicAdd(a.obs + 2 * ((size_t)j * a.n_obs + o) + (jj < a.Rp ? 0 : 1), f);
          }
        }
      }
    } else {
    float* ft = reinterpret_cast<float*>(&S.stage[0][0][0]);
    if (ok) {
#pragma unroll
      for (int c = 0; c < 64; ++c) ft[(64 * h + c) * kFStride + r] = __fmul_rn(__fadd_rn(hi[c], lo[c * kBM]), rs);
    }
    epi_bar();
    if (!*(volatile int*)&S.abort) {
      // ---- fused RK4 stage update in runs of 8 rows: lane -> (column & 7, row run & 3)
      const int u = t - 64, ew = u >> 5;
      const int nlo = lane & 7, glo = lane >> 3;
      const int s = a.stage;
      const float cst = (s == 2) ? a.c_full : a.c_half;
      bool bad = false, range = false;
#pragma unroll 1
      for (int it = 0; it < 8; ++it) {
        const int wi = it * 8 + ew;
        const int jl = (wi >> 2) * 8 + nlo;
        const int dl = ((wi & 3) * 4 + glo) * 8;
        const int jj = nt * kBN + jl, d = mt * kBM + dl;
        const size_t e = (size_t)jj * a.Dp + d;
        float f[8], ph[8], sv[8];
        ld8(ft + jl * kFStride + dl, f);
        ld8(a.Phi + e, ph);
        if (s == 0) {
          st8(a.Acc + e, f);
#pragma unroll
          for (int i = 0; i < 8; ++i) sv[i] = __fmaf_rn(cst, f[i], ph[i]);
        } else if (s < 3) {
          float ac[8];
          ld8(a.Acc + e, ac);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            ac[i] = __fmaf_rn(2.f, f[i], ac[i]);
            sv[i] = __fmaf_rn(cst, f[i], ph[i]);
          }
          st8(a.Acc + e, ac);
        } else {
          float ac[8], pl[8];
          ld8(a.Acc + e, ac);
          ld8(a.Plo + e, pl);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float ksum = __fadd_rn(ac[i], f[i]);
            const float inc = __fmul_rn(ksum, a.c_sixth);
            const float inc_res = __fmaf_rn(ksum, a.c_sixth, -inc);
            const float inc_lo = __fmaf_rn(ksum, a.c_sixth_lo, inc_res);
            const float x = ph[i];
            const float sm = __fadd_rn(x, inc);
            const float bv = __fsub_rn(sm, x);
            const float er = __fadd_rn(__fsub_rn(x, __fsub_rn(sm, bv)), __fsub_rn(inc, bv));
            float l = __fadd_rn(pl[i], __fadd_rn(er, inc_lo));
            const float h2 = __fadd_rn(sm, l);
            l = __fsub_rn(l, __fsub_rn(h2, sm));
            ph[i] = h2;
            pl[i] = l;
            sv[i] = h2;
            bad |= !isfinite(h2);
          }
          st8(a.Phi + e, ph);
          st8(a.Plo + e, pl);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          sv[i] = __fmul_rn(sv[i], a.sb);
          range |= !(fabsf(sv[i]) <= kBMax);
        }
        scatter_b8(a, d, jj, sv);
      }
      if (bad) atomicOr(a.status, LIME_FLAG_NONFINITE);
      if (range) atomicOr(a.status, LIME_FLAG_RANGE);
    }
    }
  }

  tc::tc_fence_before();
  __syncthreads();
  if (t == 0 && S.abort) atomicOr(a.status, LIME_FLAG_TIMEOUT);
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tbase, kTmemCols);
  }
}

// ---------------------------------------------------------------- set-up kernels
// A pieces of one row (row = blockIdx.x) of [Mr | Mi]: the row is scaled by
// the power of two that brings its largest component into [2^12, 2^13), then
// split as A0 = 64 k (|k| <= 127) + fp16 residuals A1, A2; row_inv gets the
// inverse scale (0 for padding rows and all-zero rows).  transposed = 0:
// M = L (D x D, element (row, kk) = L[row][kk]); transposed = 1: M = the
// observables, element (o, a n + b) = E_o[b][a], so that <E_o> = sum_d M[o][d]
// vec(rho)[d].
__global__ void convert_rows_kernel(const double2* M, int transposed, int n, int rows, int D, int Dp, int KC,
                                    uint8_t* A0, uint8_t* A1, uint8_t* A2, float* row_inv) {
  __shared__ double red[8];
  const int row = blockIdx.x;
  auto elem = [&](int kk) -> double2 {
    if (!transposed) return M[(size_t)row * D + kk];
    const int ia = kk / n, ib = kk - ia * n;
    return M[(size_t)row * D + (size_t)ib * n + ia];
  };
  double mx = 0.0;
  if (row < rows)
    for (int k = threadIdx.x; k < D; k += blockDim.x) {
      const double2 z = elem(k);
      mx = fmax(mx, fmax(fabs(z.x), fabs(z.y)));
    }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    red[0] = m;
  }
  __syncthreads();
  mx = red[0];
  int sh = 0;
  bool live = row < rows && mx > 0.0 && isfinite(mx);
  if (live) {
    sh = 12 - ilogb(mx);                 // mx * 2^sh in [2^12, 2^13)
    if (sh > 140 || sh < -140) live = false;
  }
  if (threadIdx.x == 0) row_inv[row] = live ? ldexpf(1.f, -sh) : 0.f;
  const int mt = row >> 7, rr = row & 127;
  for (int k = threadIdx.x; k < 2 * Dp; k += blockDim.x) {
    double x = 0.0;
    if (live) {
      const int kk = k < Dp ? k : k - Dp;
      if (kk < D) {
        const double2 z = elem(kk);
        x = ldexp(k < Dp ? z.x : z.y, sh);
      }
    }
    const double kq = fmin(fmax(rint(x * (1.0 / 64.0)), -kA0Max), kA0Max);
    const double v0 = kq * 64.0;
    const double r1 = x - v0;
    const __half h1 = __double2half(r1);
    const __half h2 = __double2half(r1 - (double)__half2float(h1));
    const size_t off = ((size_t)mt * KC + k / kCK) * kPiece + blk_off(rr, k % kCK);
    *reinterpret_cast<__half*>(A0 + off) = __double2half(v0);
    *reinterpret_cast<__half*>(A1 + off) = h1;
    *reinterpret_cast<__half*>(A2 + off) = h2;
  }
}

// state from complex128 rho [R][D] (row-major vec per RHS) and the first B input
__global__ void init_state_kernel(StageArgs a, const double2* rho, int D, int R) {
  const size_t total = (size_t)a.W * a.Dp;
  bool range = false;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int jj = (int)(e / a.Dp), d = (int)(e % a.Dp);
    const int j = jj < a.Rp ? jj : jj - a.Rp;
    double v = 0.0;
    if (d < D && j < R) {
      const double2 z = rho[(size_t)j * D + d];
      v = jj < a.Rp ? z.x : z.y;
    }
    const float hv = (float)v;
    a.Phi[e] = hv;
    a.Plo[e] = (float)(v - (double)hv);
    const float x = __fmul_rn(hv, a.sb);
    range |= !(fabsf(x) <= kBMax);
    scatter_b1(a, d, jj, x);
  }
  if (range) atomicOr(a.status, LIME_FLAG_RANGE);
}

__global__ void final_state_kernel(const float* Phi, const float* Plo, int Dp, int Rp, double2* rho, int D, int R) {
  const size_t total = (size_t)R * D;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / D), d = (int)(e % D);
    const size_t er = (size_t)j * Dp + d, ei = (size_t)(j + Rp) * Dp + d;
    rho[e] = make_double2((double)Phi[er] + (double)Plo[er], (double)Phi[ei] + (double)Plo[ei]);
  }
}

}  // namespace rsp
}  // namespace lime

using namespace lime;

static void rsp_dims(int n, int R, int& D, int& Dp, int& Rp, int& W, int& KC, int& MT, int& NT) {
  D = n * n;
  Dp = (D + 127) / 128 * 128;
  Rp = (R + 63) / 64 * 64;
  W = 2 * Rp;
  KC = 2 * Dp / rsp::kCK;
  MT = Dp / 128;
  NT = W / 128;
}

struct RspLayout {
  size_t apiece, epiece, bpiece, state, rows;
  size_t total;
};

static RspLayout rsp_layout(int n, int R, int n_obs) {
  int D, Dp, Rp, W, KC, MT, NT;
  rsp_dims(n, R, D, Dp, Rp, W, KC, MT, NT);
  const int MTo = n_obs > 0 ? (n_obs + 127) / 128 : 0;
  RspLayout l;
  l.apiece = (size_t)MT * KC * rsp::kPiece;
  l.epiece = (size_t)MTo * KC * rsp::kPiece;
  l.bpiece = (size_t)NT * KC * rsp::kPiece;
  l.state = (size_t)W * Dp * sizeof(float);
  l.rows = (size_t)(MT + MTo) * 128 * sizeof(float);
  l.total = 3 * l.apiece + 3 * l.epiece + 4 * l.bpiece + 3 * l.state + ((l.rows + 1023) / 1024) * 1024 + 4096;
  return l;
}

extern "C" size_t lime_redfield_split_workspace(int32_t n, int32_t n_rhs, int32_t n_obs) {
  if (n <= 0 || n_rhs <= 0 || n_obs < 0) return 0;
  return rsp_layout(n, n_rhs, n_obs).total;
}

extern "C" int lime_redfield_rk4_split(const LimeRedfieldSplitDesc* d, void* stream) {
  if (!d || d->n <= 0 || d->n_rhs <= 0 || d->n_steps < 0 || d->n_obs < 0) return LIME_ERR_ARG;
  if (!d->R || !d->rho || !d->workspace || !d->status) return LIME_ERR_ARG;
  if (d->n_obs > 0 && (!d->obs_ops || !d->obs_out)) return LIME_ERR_ARG;
  if (d->scale_b_log2 < -60 || d->scale_b_log2 > 60) return LIME_ERR_ARG;
  if ((int64_t)d->n * d->n > (1 << 20)) return LIME_ERR_UNSUPPORTED;
  if (d->workspace_bytes < lime_redfield_split_workspace(d->n, d->n_rhs, d->n_obs)) return LIME_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(d->workspace) & 1023) != 0) return LIME_ERR_ARG;
  int D, Dp, Rp, W, KC, MT, NT;
  rsp_dims(d->n, d->n_rhs, D, Dp, Rp, W, KC, MT, NT);
  const int MTo = d->n_obs > 0 ? (d->n_obs + 127) / 128 : 0;
  const RspLayout L = rsp_layout(d->n, d->n_rhs, d->n_obs);
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* ws = reinterpret_cast<uint8_t*>(d->workspace);
  uint8_t* A[3] = {ws, ws + L.apiece, ws + 2 * L.apiece};
  uint8_t* Ep[3] = {ws + 3 * L.apiece, ws + 3 * L.apiece + L.epiece, ws + 3 * L.apiece + 2 * L.epiece};
  uint8_t* bb = ws + 3 * L.apiece + 3 * L.epiece;
  uint8_t* B[4] = {bb, bb + L.bpiece, bb + 2 * L.bpiece, bb + 3 * L.bpiece};
  float* Phi = reinterpret_cast<float*>(bb + 4 * L.bpiece);
  float* Plo = Phi + (size_t)W * Dp;
  float* Acc = Plo + (size_t)W * Dp;
  float* row_inv = Acc + (size_t)W * Dp;           // [MT*128] generator rows, then [MTo*128] observables
  int64_t launches = 0;

  rsp::convert_rows_kernel<<<Dp, 256, 0, st>>>(reinterpret_cast<const double2*>(d->R), 0, d->n, D, D, Dp, KC,
                                              A[0], A[1], A[2], row_inv);
  LIME_CUDA_TRY(cudaGetLastError());
  ++launches;
  if (MTo > 0) {
    rsp::convert_rows_kernel<<<MTo * 128, 256, 0, st>>>(reinterpret_cast<const double2*>(d->obs_ops), 1, d->n,
                                                       d->n_obs, D, Dp, KC, Ep[0], Ep[1], Ep[2],
                                                       row_inv + (size_t)MT * 128);
    LIME_CUDA_TRY(cudaGetLastError());
    ++launches;
    const int obs_every = d->obs_every > 0 ? d->obs_every : 1;
    const size_t slots = (size_t)(d->n_steps / obs_every);
    if (slots > 0) {
      LIME_CUDA_TRY(cudaMemsetAsync(d->obs_out, 0, slots * d->n_rhs * d->n_obs * 2 * sizeof(double), st));
    }
  }

  rsp::StageArgs a{};
  a.Dp = Dp; a.W = W; a.KC = KC; a.MT = MT; a.NT = NT; a.Rp = Rp; a.R = d->n_rhs;
  a.KS = 1; a.groups_per_split = KC / rsp::kGroup;
  a.inv_sb = ldexpf(1.f, -d->scale_b_log2);
  a.sb = ldexpf(1.f, d->scale_b_log2);
  a.magic_b = ldexpf(1.5f, 23 + 3);          // B0 quantum q_B = 2^3 (|B| <= 2^13)
  a.c_half = (float)(d->dt / 2.0);
  a.c_full = (float)d->dt;
  a.c_sixth = (float)(d->dt / 6.0);
  a.c_sixth_lo = (float)(d->dt / 6.0 - (double)a.c_sixth);
  a.A[0] = A[0]; a.A[1] = A[1]; a.A[2] = A[2];
  a.row_inv = row_inv;
  a.Phi = Phi; a.Plo = Plo; a.Acc = Acc;
  a.status = d->status;
  a.max_wait = 1u << 26;
  // first B input = rho0
  a.Bn[0] = B[0]; a.Bn[1] = B[1];
  const size_t tot = (size_t)W * Dp;
  const int ib = (int)((tot + 255) / 256);
  rsp::init_state_kernel<<<ib < 65535 ? ib : 65535, 256, 0, st>>>(a, reinterpret_cast<const double2*>(d->rho), D,
                                                                   d->n_rhs);
  LIME_CUDA_TRY(cudaGetLastError());
  ++launches;

  // observable pass: same operands as a stage with A = observables, K split
  // so that the grid covers the GPU about twice
  rsp::StageArgs ao = a;
  int n_sm = 148;
  {
    int dev = 0;
    LIME_CUDA_TRY(cudaGetDevice(&dev));
    LIME_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
  }
  if (MTo > 0) {
    ao.MT = MTo;
    ao.A[0] = Ep[0]; ao.A[1] = Ep[1]; ao.A[2] = Ep[2];
    ao.row_inv = row_inv + (size_t)MT * 128;
    ao.n_obs = d->n_obs;
    const int groups = KC / rsp::kGroup;
    int ks = (2 * n_sm) / (MTo * NT);
    ks = ks < 1 ? 1 : (ks > groups ? groups : ks);
    ao.groups_per_split = (groups + ks - 1) / ks;
    ao.KS = (groups + ao.groups_per_split - 1) / ao.groups_per_split;
  }

  const size_t smem = sizeof(rsp::Smem) + 1024;
  LIME_CUDA_TRY(cudaFuncSetAttribute(rsp::gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  LIME_CUDA_TRY(cudaFuncSetAttribute(rsp::gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int obs_every = d->obs_every > 0 ? d->obs_every : 1;
  int cur = 0;   // B[2cur], B[2cur+1] hold the current stage input
  for (int step = 0; step < d->n_steps; ++step) {
    for (int s = 0; s < 4; ++s) {
      a.stage = s;
      a.Bc[0] = B[2 * cur]; a.Bc[1] = B[2 * cur + 1];
      a.Bn[0] = B[2 * (cur ^ 1)]; a.Bn[1] = B[2 * (cur ^ 1) + 1];
      rsp::gemm_kernel<false><<<MT * NT, rsp::kThreads, smem, st>>>(a);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
      cur ^= 1;
    }
    if (MTo > 0 && ((step + 1) % obs_every) == 0) {
      // B[2cur], B[2cur+1] now hold the new state (the next step's stage-0 input)
      const int slot = (step + 1) / obs_every - 1;
      ao.Bc[0] = B[2 * cur]; ao.Bc[1] = B[2 * cur + 1];
      ao.obs = d->obs_out + (size_t)slot * d->n_rhs * d->n_obs * 2;
      rsp::gemm_kernel<true><<<ao.KS * MTo * NT, rsp::kThreads, smem, st>>>(ao);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
    }
  }
  const int fb = (int)(((size_t)d->n_rhs * D + 255) / 256);
  rsp::final_state_kernel<<<fb < 65535 ? fb : 65535, 256, 0, st>>>(Phi, Plo, Dp, Rp,
                                                                     reinterpret_cast<double2*>(d->rho), D, d->n_rhs);
  LIME_CUDA_TRY(cudaGetLastError());
  ++launches;
  count_launch(launches);
  return LIME_OK;
}
