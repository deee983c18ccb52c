// Streaming split-precision GEMM tile on the sm_103a tensor cores (tcgen05),
// shared by the dense Redfield RK4 and the general (dense collapse operator)
// Lindblad RK4.
//
// One CTA computes one 128 x 128 fp32 tile of the real product C = A . B
// where both operands live in global memory pre-tiled in the canonical
// K-major, no-swizzle UMMA layout: every (128-row tile, 64-wide K chunk)
// block is one contiguous 16 KB piece (blk_off), moved by the bulk-copy
// (TMA) engine with cp.async.bulk into a two-stage shared-memory ring and
// completed on mbarriers (two 64-K stages measured faster than four 32-K
// ones).
//
// Warp roles (64 + 32 kEpiWarps threads, 1 CTA/SM):
//   warp 0      producer: bulk copies of 5 pieces per K chunk (80 KB)
//   warp 1      MMA issuer: tcgen05.mma M=128 N=128 K=16, kind::f16
//   warps 2..17 epilogue: drain TMEM accumulators into fp32 two-sum
//               accumulators (hi words in registers, lo words in shared
//               memory), then park the finished tile in shared memory for
//               the caller's fused epilogue.
//
// Precision.  A = A0 (per-row 7-bit fixed point, 64 k with |k| <= 127 after
// the row's power-of-two scaling) + A1 + A2 (fp16 residuals); B = B0
// (10-bit fixed point, quantum 8 after the operand's power-of-two scaling)
// + B1 (fp16 residual).  A tcgen05.mma rounds its fp32 result toward zero,
// so the dominant product A0.B0 is kept exact: it is accumulated over 128 K
// (integer multiples of 512 below 2^24) in its own TMEM accumulator D0, the
// small products A1.B0 + A0.B1 + A1.B1 + A2.B0 in D1; every 128 K D0 enters
// an fp32 two-sum (hi, lo) and D1 is added to lo, round to nearest.  TMEM:
// D0/D1 double buffered, 4 x 128 = 512 columns, so the MMAs of the next
// 128 K overlap the promotion of the previous ones.
#pragma once

#include "common.cuh"
#include "tc_ptx.cuh"

namespace lime {
namespace sg {

constexpr int kBM = 128, kBN = 128;                // output tile
constexpr int kCK = 64;                            // K per chunk (one ring stage)
constexpr int kGroup = 128 / kCK;                  // chunks per exactly accumulated 128 K
constexpr uint32_t kPiece = 128 * kCK * 2;         // 128 x 64 fp16 = 16 KB
constexpr int kStages = 2;
// epilogue warps: 4 TMEM lane quadrants x column groups.  16 (32 columns a
// thread, 96 registers) measured 4.8 % faster than 8 (64 columns, 168
// registers) on the 9216-dim Redfield stage and 4 % on the uneven batch.
constexpr int kEpiWarps = 16;
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kThreads = 64 + kEpiThreads;         // + producer warp + MMA warp
constexpr int kEpiCols = kBN / (kEpiWarps / 4);    // tile columns per epilogue thread
constexpr int kEpiFirst = 64;                      // first epilogue thread
constexpr uint32_t kLBO = 128, kSBO = kCK * 16;    // canonical K-major block strides (bytes)
constexpr uint32_t kTmemCols = 512;
constexpr double kA0Max = 127.0;
constexpr float kBMax = 8192.f;                    // |B| bound of the 10-bit fixed point (quantum 8)
constexpr float kMagicB = 1.5f * 8388608.f * 8.f;  // 1.5 * 2^23 * 8: (x + M) - M rounds x to a multiple of 8
constexpr int kFStride = kBN + 4;                  // padded column of the parked tile (floats)

// The epilogue's index arithmetic holds only for these shapes.  Each column
// group is drained by four warps (one per TMEM lane quadrant: a warp may
// only read its own 32 lanes), 16 columns per tcgen05.ld, and the groups
// must tile the accumulator exactly: a width that over-covers it (three
// groups of 48 columns for a 12-warp epilogue: 144 > 128) reads TMEM columns
// past the allocation (D1 of the second buffer at 2*128 + 128 + 96 + 47 =
// 527 > 511) and writes the two-sum words past S.lo, over the barriers and
// beyond the dynamic shared allocation: an illegal address.
static_assert(kEpiWarps % 4 == 0, "a column group needs one warp per TMEM lane quadrant");
static_assert(kEpiCols % 16 == 0, "the drain reads 16 accumulator columns per tcgen05.ld");
static_assert(kEpiCols * (kEpiWarps / 4) == kBN, "the column groups must tile the tile's columns exactly");
static_assert(2 * 2 * kBN <= (int)kTmemCols, "D0 and D1, double-buffered, must fit the TMEM allocation");
static_assert(kBM == 128, "one accumulator row per TMEM lane");
static_assert(kThreads <= 1024, "one CTA");
static_assert(kCK % 16 == 0 && 128 % kCK == 0, "K chunks are whole MMA K steps and divide the exact group");

struct __align__(1024) Smem {
  uint8_t stage[kStages][5][kPiece];               // A0 A1 A2 B0 B1; the parked tile after the last MMA
  float lo[kBN * kBM];                             // low words of the fp32 two-sum accumulators, [col][row]
  uint64_t full[kStages], empty[kStages], accf[2], acce[2], drain;
  uint32_t tmem_base;
  int abort;
  __device__ float* tile() { return reinterpret_cast<float*>(&stage[0][0][0]); }   // [col][row], stride kFStride
};
static_assert((size_t)kBN * kFStride * sizeof(float) <= sizeof(Smem::stage), "parked tile fits the ring");
constexpr size_t kSmemBytes = sizeof(Smem) + 1024;

// byte offset of (row, k) inside one 128 x kCK block
__host__ __device__ __forceinline__ uint32_t blk_off(int row, int k) {
  return (uint32_t)(row >> 3) * kSBO + (uint32_t)(k >> 3) * kLBO + (uint32_t)(row & 7) * 16u +
         (uint32_t)(k & 7) * 2u;
}
// byte offset of (row, k) in an operand of KC chunks per 128-row tile
__host__ __device__ __forceinline__ size_t piece_off(int KC, int row, int k) {
  return ((size_t)(row >> 7) * KC + k / kCK) * kPiece + blk_off(row & 127, k % kCK);
}

// x (scaled) = v0 (multiple of 8) + v1
__device__ __forceinline__ void split_b(float x, float& v0, float& v1) {
  v0 = __fsub_rn(__fadd_rn(x, kMagicB), kMagicB);
  v1 = __fsub_rn(x, v0);
}

// 8 scaled B values at (row n, k..k+7), k % 8 == 0, as two 16-byte stores
// per piece; `neg` stores their negatives.  avail: bytes of each piece
// buffer from B0 / B1 (checked in the bounds-checked build).
__device__ __forceinline__ void store_b8(uint8_t* B0, uint8_t* B1, int KC, int n, int k, const float (&x)[8],
                                         bool neg, size_t avail = kNoExtent, int32_t* status = nullptr) {
  uint32_t h0[4], h1[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float a0, a1, b0, b1;
    split_b(x[2 * i], a0, a1);
    split_b(x[2 * i + 1], b0, b1);
    const __half2 p = __floats2half2_rn(a0, b0);
    const __half2 q = __floats2half2_rn(a1, b1);
    h0[i] = *reinterpret_cast<const uint32_t*>(&p);
    h1[i] = *reinterpret_cast<const uint32_t*>(&q);
  }
  const uint32_t sg = neg ? 0x80008000u : 0u;
  const size_t off = piece_off(KC, n, k);
  if (!in_bounds(off, 16, avail, status)) return;
  *reinterpret_cast<uint4*>(B0 + off) = make_uint4(h0[0] ^ sg, h0[1] ^ sg, h0[2] ^ sg, h0[3] ^ sg);
  *reinterpret_cast<uint4*>(B1 + off) = make_uint4(h1[0] ^ sg, h1[1] ^ sg, h1[2] ^ sg, h1[3] ^ sg);
}

// Complex matrix S (K x N) into the real block operand [[Sr, Si], [-Si, Sr]]
// (2K x 2N), stored transposed (B^T rows = the 2N output columns, K-major):
// 8 consecutive rows k..k+7 of column j of S, real (im = false) or
// imaginary parts, scaled.  Kp, Np: padded K and N (row/column offsets of
// the second block).
__device__ __forceinline__ void scatter_cplx8(uint8_t* B0, uint8_t* B1, int KC, int Kp, int Np, int k, int j,
                                              bool im, const float (&x)[8], size_t avail = kNoExtent,
                                              int32_t* status = nullptr) {
  if (!im) {
    store_b8(B0, B1, KC, j, k, x, false, avail, status);             // Sr at (k, j)
    store_b8(B0, B1, KC, j + Np, Kp + k, x, false, avail, status);   // Sr at (K + k, N + j)
  } else {
    store_b8(B0, B1, KC, j, Kp + k, x, true, avail, status);         // -Si at (K + k, j)
    store_b8(B0, B1, KC, j + Np, k, x, false, avail, status);        // Si at (k, N + j)
  }
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

// RK4 constants of one stage
struct RK4 {
  int stage;                                      // 0..3
  float c_half, c_full, c_sixth, c_sixth_lo;      // dt/2, dt, dt/6 = c_sixth + c_sixth_lo
};

// One RK4 stage (lime/phys.py:636-649) for 8 state elements at e..e+7 of
// the planar fp32 state (Phi + Plo, accumulator Acc) with derivative f:
// writes the next stage input to sv (the new state after stage 3).
__device__ __forceinline__ void rk4_stage8(const RK4& k, float* Phi, float* Plo, float* Acc, size_t e,
                                           const float (&f)[8], float (&sv)[8], bool& bad) {
  float ph[8];
  ld8(Phi + e, ph);
  const int s = k.stage;
  const float cst = (s == 2) ? k.c_full : k.c_half;
  if (s == 0) {
    st8(Acc + e, f);
#pragma unroll
    for (int i = 0; i < 8; ++i) sv[i] = __fmaf_rn(cst, f[i], ph[i]);
  } else if (s < 3) {
    float ac[8];
    ld8(Acc + e, ac);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      ac[i] = __fmaf_rn(2.f, f[i], ac[i]);
      sv[i] = __fmaf_rn(cst, f[i], ph[i]);
    }
    st8(Acc + e, ac);
  } else {
    float ac[8], pl[8];
    ld8(Acc + e, ac);
    ld8(Plo + e, pl);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      ph[i] = rk4_final_f32(ph[i], ac[i], f[i], k.c_sixth, k.c_sixth_lo, pl[i]);
      sv[i] = ph[i];
      bad |= !isfinite(ph[i]);
    }
    st8(Phi + e, ph);
    st8(Plo + e, pl);
  }
}

__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory"); }

// The operands and scaling of one tile.
struct Tile {
  const uint8_t* A[3];     // A pieces of this tile's 128-row block, chunk 0 (chunk c at + c * kPiece)
  const uint8_t* B[2];     // B pieces of this tile's 128-column block, chunk 0
  int c0, n_chunks;        // chunk range [c0, c0 + n_chunks), n_chunks a multiple of kGroup
  const float* row_inv;    // 128 per-row inverse A scales of the tile (0 on padding rows)
  float inv_sb;            // inverse B scale
  uint32_t max_wait;       // bound on every mbarrier poll loop
  int withhold = 0;        // self-test only: the producer issues no copies, so every wait expires
  // bytes readable from A[i] / B[i] (checked in the bounds-checked build:
  // a chunk past them is not copied, and the tile aborts)
  size_t a_avail = kNoExtent, b_avail = kNoExtent;
  int32_t* status = nullptr;
  // park the two-sum words separately (mainloop): hi * scale into the ring
  // tile, lo * scale in place in S.lo ([col][row], stride kBM), for callers
  // that combine tiles with cancellation
  int park_split = 0;
};

// TMEM allocation and barrier set-up; every thread of the CTA calls it.
__device__ __forceinline__ void setup(Smem& S) {
  const int t = threadIdx.x, warp = t >> 5;
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
}

// Every thread: waits for the CTA, raises LIME_FLAG_TIMEOUT if a wait
// expired, releases TMEM.
__device__ __forceinline__ void teardown(Smem& S, int32_t* status) {
  tc::tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0 && S.abort) atomicOr(status, LIME_FLAG_TIMEOUT);
  if ((threadIdx.x >> 5) == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(S.tmem_base, kTmemCols);
  }
}

// The tile's main loop.  Returns true on the kEpiThreads epilogue threads, which on
// return have parked C[r][c] * row_inv[r] * inv_sb at S.tile()[c * kFStride
// + r] and passed a named barrier together (unless S.abort is set: a wait
// expired and the tile is not valid); false on the producer and MMA warps.
__device__ __forceinline__ bool mainloop(Smem& S, const Tile& T) {
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const uint32_t tbase = S.tmem_base;
  const int KC = T.n_chunks;

  if (warp == 0) {
    // ---------------- producer
    if (lane == 0) {
      int issued = 0;
      for (int c = 0; c < KC; ++c) {
        const int s = c % kStages;
        const uint32_t ph = (uint32_t)(c / kStages) & 1u;
        if (!tc::mbar_wait_bounded(&S.empty[s], ph ^ 1u, T.max_wait)) { atomicExch(&S.abort, 1); break; }
        if (*(volatile int*)&S.abort || T.withhold) break;
        if (!in_bounds((size_t)(T.c0 + c) * kPiece, kPiece, T.a_avail, T.status) ||
            !in_bounds((size_t)(T.c0 + c) * kPiece, kPiece, T.b_avail, T.status)) {
          atomicExch(&S.abort, 1);
          break;
        }
        issued = c + 1;
        tc::mbar_arrive_expect_tx(&S.full[s], 5 * kPiece);
        const size_t off = (size_t)(T.c0 + c) * kPiece;
        tc::bulk_g2s(S.stage[s][0], T.A[0] + off, kPiece, &S.full[s]);
        tc::bulk_g2s(S.stage[s][1], T.A[1] + off, kPiece, &S.full[s]);
        tc::bulk_g2s(S.stage[s][2], T.A[2] + off, kPiece, &S.full[s]);
        tc::bulk_g2s(S.stage[s][3], T.B[0] + off, kPiece, &S.full[s]);
        tc::bulk_g2s(S.stage[s][4], T.B[1] + off, kPiece, &S.full[s]);
      }
      // the copies of the last (up to kStages) issued chunks have landed before exit
      for (int c = issued - 1; c >= 0 && c >= issued - kStages; --c)
        tc::mbar_wait_bounded(&S.full[c % kStages], (uint32_t)(c / kStages) & 1u, T.max_wait);
    }
    return false;
  }
  if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_f16(kBM, kBN, 0);
      for (int c = 0; c < KC; ++c) {
        const int s = c % kStages;
        const uint32_t ph = (uint32_t)(c / kStages) & 1u;
        const int p = c / kGroup, b = p & 1;
        const bool first = (c % kGroup) == 0;
        const bool last = (c % kGroup) == kGroup - 1;
        if (!tc::mbar_wait_bounded(&S.full[s], ph, T.max_wait)) { atomicExch(&S.abort, 1); break; }
        if (first && !tc::mbar_wait_bounded(&S.acce[b], ((uint32_t)(p >> 1) & 1u) ^ 1u, T.max_wait)) {
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
      tc::mbar_wait_bounded(&S.drain, 0u, T.max_wait);
    }
    return false;
  }

  // ---------------- epilogue: 8 warps, TMEM lane quadrant warp & 3, column half
  const int lq = warp & 3;
  const int h = (warp - 2) >> 2;                  // column group of kEpiCols
  const int r = lq * 32 + lane;
  const uint32_t lane_addr = tbase + ((uint32_t)(lq * 32) << 16);
  // hi words in registers, lo words in shared memory (each thread owns its
  // 64 entries; lanes hit consecutive words)
  float hi[kEpiCols];
  float* lo = S.lo + (kEpiCols * h) * kBM + r;
#pragma unroll
  for (int c = 0; c < kEpiCols; ++c) { hi[c] = 0.f; lo[c * kBM] = 0.f; }
  const int n_groups = KC / kGroup;
  bool ok = true;
  for (int p = 0; p < n_groups; ++p) {
    const int b = p & 1;
    if (!tc::mbar_wait_bounded(&S.accf[b], (uint32_t)(p >> 1) & 1u, T.max_wait)) {
      atomicExch(&S.abort, 1);
      ok = false;
      break;
    }
    tc::tc_fence_after();
    const uint32_t d0 = lane_addr + (uint32_t)(2 * b) * 128u + (uint32_t)(kEpiCols * h);
#pragma unroll
    for (int q = 0; q < kEpiCols / 16; ++q) {
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
  // park the tile in the ring: every MMA has completed once the last
  // accumulator group was seen, so the tensor core reads no operand
  const float rs = __fmul_rn(T.row_inv[r], T.inv_sb);
  float* ft = S.tile();
  if (ok) {
    if (T.park_split) {
#pragma unroll
      for (int c = 0; c < kEpiCols; ++c) {
        ft[(kEpiCols * h + c) * kFStride + r] = __fmul_rn(hi[c], rs);
        lo[c * kBM] = __fmul_rn(lo[c * kBM], rs);
      }
    } else {
#pragma unroll
      for (int c = 0; c < kEpiCols; ++c)
        ft[(kEpiCols * h + c) * kFStride + r] = __fmul_rn(__fadd_rn(hi[c], lo[c * kBM]), rs);
    }
  }
  epi_bar();
  return true;
}

// ---------------------------------------------------------------- tile sequences
// A persistent CTA runs a sequence of tiles in one launch and keeps the
// ring, the TMEM accumulators and their barriers from tile to tile: the
// chunk counter gc and the accumulator-group counter gp run on across
// tiles, so the producer and the MMA issuer start the next tile's copies and
// its first two 128-K groups (the double-buffered D0/D1) while the epilogue
// warps are still in the previous tile's fused epilogue.  The finished tile
// is parked in place in the two-sum buffer S.lo (the ring by then holds the
// next tile's operands), in a swizzled layout (park_idx): a drain writes 32
// consecutive rows of one column per warp, a fused epilogue reads 8-row runs
// of 8 columns, both without bank conflicts.
struct Seq {
  int gc = 0;   // chunks issued (producer) / consumed (MMA issuer) so far
  int gp = 0;   // 128-K accumulator groups committed (MMA issuer) / drained (epilogue) so far
};

__host__ __device__ __forceinline__ int park_idx(int col, int row) { return col * kBM + (row ^ ((col & 7) << 2)); }

// parked rows row..row+7 (row % 8 == 0) of column col
__device__ __forceinline__ void ld8_park(const float* ft, int col, int row, float (&v)[8]) {
  const int sw = (col & 7) << 2;
  const float4 x = *reinterpret_cast<const float4*>(ft + col * kBM + (row ^ sw));
  const float4 y = *reinterpret_cast<const float4*>(ft + col * kBM + ((row + 4) ^ sw));
  v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w; v[4] = y.x; v[5] = y.y; v[6] = y.z; v[7] = y.w;
}

// named barrier of the epilogue warps that also ORs a predicate over them
__device__ __forceinline__ bool epi_bar_or(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "barrier.cta.red.or.pred q, 1, %2, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(kEpiThreads)
      : "memory");
  return r != 0;
}

// bounded wait that also gives up once another role of the CTA has aborted
// (checked every 256 polls), so one expired wait ends the whole sequence
__device__ __forceinline__ bool seq_wait(Smem& S, uint64_t* bar, uint32_t parity, uint32_t max_iters) {
  for (uint32_t it = 0; it < max_iters; ++it) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u && *(volatile int*)&S.abort) return false;
  }
  return false;
}

// producer (warp 0, lane 0): the bulk copies of the tile's chunks.  False
// once the CTA aborts (a wait expired, or a chunk past an operand's extent).
__device__ __forceinline__ bool seq_produce(Smem& S, const Tile& T, Seq& q) {
  for (int c = 0; c < T.n_chunks; ++c, ++q.gc) {
    const int s = q.gc % kStages;
    const uint32_t ph = (uint32_t)(q.gc / kStages) & 1u;
    if (!seq_wait(S, &S.empty[s], ph ^ 1u, T.max_wait)) { atomicExch(&S.abort, 1); return false; }
    if (*(volatile int*)&S.abort) return false;
    if (!in_bounds((size_t)(T.c0 + c) * kPiece, kPiece, T.a_avail, T.status) ||
        !in_bounds((size_t)(T.c0 + c) * kPiece, kPiece, T.b_avail, T.status)) {
      atomicExch(&S.abort, 1);
      return false;
    }
    tc::mbar_arrive_expect_tx(&S.full[s], 5 * kPiece);
    const size_t off = (size_t)(T.c0 + c) * kPiece;
    tc::bulk_g2s(S.stage[s][0], T.A[0] + off, kPiece, &S.full[s]);
    tc::bulk_g2s(S.stage[s][1], T.A[1] + off, kPiece, &S.full[s]);
    tc::bulk_g2s(S.stage[s][2], T.A[2] + off, kPiece, &S.full[s]);
    tc::bulk_g2s(S.stage[s][3], T.B[0] + off, kPiece, &S.full[s]);
    tc::bulk_g2s(S.stage[s][4], T.B[1] + off, kPiece, &S.full[s]);
  }
  return true;
}

// producer, after its last tile: the copies still in flight have landed
__device__ __forceinline__ void seq_produce_end(Smem& S, const Seq& q, uint32_t max_wait) {
  for (int c = q.gc - 1; c >= 0 && c >= q.gc - kStages; --c)
    tc::mbar_wait_bounded(&S.full[c % kStages], (uint32_t)(c / kStages) & 1u, max_wait);
}

// MMA issuer (warp 1, lane 0): the tile's MMAs, one accumulator group per
// 128 K into D0/D1 buffer gp & 1.
__device__ __forceinline__ bool seq_mma(Smem& S, const Tile& T, Seq& q) {
  constexpr uint32_t idesc = tc::idesc_f16(kBM, kBN, 0);
  const uint32_t tbase = S.tmem_base;
  for (int c = 0; c < T.n_chunks; ++c, ++q.gc) {
    const int s = q.gc % kStages;
    const uint32_t ph = (uint32_t)(q.gc / kStages) & 1u;
    const int b = q.gp & 1;
    const bool first = (c % kGroup) == 0;
    const bool last = (c % kGroup) == kGroup - 1;
    if (!seq_wait(S, &S.full[s], ph, T.max_wait)) { atomicExch(&S.abort, 1); return false; }
    if (first && !seq_wait(S, &S.acce[b], ((uint32_t)(q.gp >> 1) & 1u) ^ 1u, T.max_wait)) {
      atomicExch(&S.abort, 1);
      return false;
    }
    if (*(volatile int*)&S.abort) return false;
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
    if (last) {
      tc::mma_commit(&S.accf[b]);
      ++q.gp;
    }
  }
  return true;
}

// MMA issuer, after its last tile: every MMA has completed before TMEM is released
__device__ __forceinline__ void seq_mma_end(Smem& S, uint32_t max_wait) {
  tc::mma_commit(&S.drain);
  tc::mbar_wait_bounded(&S.drain, 0u, max_wait);
}

// epilogue warps: drain the tile's accumulator groups into the fp32 two-sum
// and park C[r][c] * row_inv[r] * inv_sb at S.lo[park_idx(c, r)]; ends with
// a named barrier of the epilogue warps.  The caller must have passed an
// epilogue barrier after reading the previous parked tile.  False if a wait
// expired (the tile is not valid).
__device__ __forceinline__ bool seq_drain(Smem& S, const Tile& T, Seq& q) {
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int lq = warp & 3;
  const int h = (warp - 2) >> 2;
  const int r = lq * 32 + lane;
  const uint32_t lane_addr = S.tmem_base + ((uint32_t)(lq * 32) << 16);
  float hi[kEpiCols];
#pragma unroll
  for (int c = 0; c < kEpiCols; ++c) {
    hi[c] = 0.f;
    S.lo[park_idx(kEpiCols * h + c, r)] = 0.f;
  }
  const int n_groups = T.n_chunks / kGroup;
  bool ok = true;
  for (int p = 0; p < n_groups; ++p, ++q.gp) {
    const int b = q.gp & 1;
    if (!seq_wait(S, &S.accf[b], (uint32_t)(q.gp >> 1) & 1u, T.max_wait)) {
      atomicExch(&S.abort, 1);
      ok = false;
      break;
    }
    tc::tc_fence_after();
    const uint32_t d0 = lane_addr + (uint32_t)(2 * b) * 128u + (uint32_t)(kEpiCols * h);
#pragma unroll
    for (int qq = 0; qq < kEpiCols / 16; ++qq) {
      float v[16], er[16];
      tc::tmem_ld16(d0 + 16 * qq, v);
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const float x = v[e];
        const float sm = __fadd_rn(hi[16 * qq + e], x);
        const float bv = __fsub_rn(sm, hi[16 * qq + e]);
        er[e] = __fadd_rn(__fsub_rn(hi[16 * qq + e], __fsub_rn(sm, bv)), __fsub_rn(x, bv));
        hi[16 * qq + e] = sm;
      }
      tc::tmem_ld16(d0 + 128u + 16 * qq, v);
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        float* l = S.lo + park_idx(kEpiCols * h + 16 * qq + e, r);
        *l = __fadd_rn(*l, __fadd_rn(er[e], v[e]));
      }
    }
    tc::tc_fence_before();
    tc::mbar_arrive(&S.acce[b]);
  }
  if (ok) {
    const float rs = __fmul_rn(T.row_inv[r], T.inv_sb);
#pragma unroll
    for (int c = 0; c < kEpiCols; ++c) {
      float* l = S.lo + park_idx(kEpiCols * h + c, r);
      *l = __fmul_rn(__fadd_rn(hi[c], *l), rs);
    }
  }
  epi_bar();
  return ok;
}

// ---------------------------------------------------------------- operand conversion
// A pieces of one row of a real operand whose K entries are value(k), k in
// [0, Ktot) (zero where the operand is padded).  The row is scaled by the
// power of two that brings its largest entry into [2^12, 2^13) and split as
// A0 = 64 k (|k| <= 127) + fp16 residuals A1, A2; row_inv gets the inverse
// scale (0 for padding rows and all-zero rows).  KC: chunks per row tile.
template <class Val>
__device__ __forceinline__ void convert_row_values(const Val& value, int row, bool valid, int Ktot, int KC,
                                                   uint8_t* A0, uint8_t* A1, uint8_t* A2, float* row_inv) {
  __shared__ double red[32];
  double mx = 0.0;
  if (valid)
    for (int k = threadIdx.x; k < Ktot; k += blockDim.x) mx = fmax(mx, fabs(value(k)));
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
  bool live = valid && mx > 0.0 && isfinite(mx);
  if (live) {
    sh = 12 - ilogb(mx);                 // mx * 2^sh in [2^12, 2^13)
    if (sh > 140 || sh < -140) live = false;
  }
  if (threadIdx.x == 0) row_inv[row] = live ? ldexpf(1.f, -sh) : 0.f;
  for (int k = threadIdx.x; k < Ktot; k += blockDim.x) {
    const double x = live ? ldexp(value(k), sh) : 0.0;
    const double kq = fmin(fmax(rint(x * (1.0 / 64.0)), -kA0Max), kA0Max);
    const double v0 = kq * 64.0;
    const double r1 = x - v0;
    const __half h1 = __double2half(r1);
    const __half h2 = __double2half(r1 - (double)__half2float(h1));
    const size_t off = piece_off(KC, row, k);
    *reinterpret_cast<__half*>(A0 + off) = __double2half(v0);
    *reinterpret_cast<__half*>(A1 + off) = h1;
    *reinterpret_cast<__half*>(A2 + off) = h2;
  }
}

// A pieces of one row of the real block row [Mr | Mi] of a complex matrix M
// (element (row, kk) read by elem, kk < cols; columns kk >= cols are zero;
// Kp is the padded column count, where the imaginary block starts).
template <class Elem>
__device__ __forceinline__ void convert_row(const Elem& elem, int row, bool valid, int cols, int Kp, int KC,
                                            uint8_t* A0, uint8_t* A1, uint8_t* A2, float* row_inv) {
  auto value = [&](int k) -> double {
    const int kk = k < Kp ? k : k - Kp;
    if (kk >= cols) return 0.0;
    const double2 z = elem(kk);
    return k < Kp ? z.x : z.y;
  };
  convert_row_values(value, row, valid, 2 * Kp, KC, A0, A1, A2, row_inv);
}

}  // namespace sg
}  // namespace lime
