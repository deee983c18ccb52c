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
// Epilogue (8 warps; thread (r, h) owns TMEM lane r, i.e. row r of [Xr; Xi],
// columns [32 h, 32 h + 32)):
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
//
// Drive (template kDrive).  Heff(t) = Heff - sum_d c_d(t) mu_d, with c_d
// held through the four stages of a step (lime/oqs.py:1691-1800): the A
// operand is split again at the start of every step, from fp32 hi/lo pairs
// of Heff, mu_d and c_d (prepared once per call in the workspace) in
// double-float arithmetic (~46 bits, FP64 being slow on this part), with
// each row's fixed-point quantum taken once from a bound of the row over
// the whole drive (max |Heff row| + sum_d max_t |c_d| max |mu_d row|).
//
// Units.  Each thread keeps its state component already in B units
// (R = +-2^b rho, the sign of the B^T row it writes) and its RK4 sums in
// accumulator units (X = 2^(a+b) Heff rho): the conversion factors are powers
// of two folded into dt/2, dt and dt/6, so the epilogue multiplies by no scale
// and the results are those of the natural-unit arithmetic scaled exactly.

#include "common.cuh"
#include "fpconv.cuh"
#include "tc_ptx.cuh"

namespace lime {
namespace split {

constexpr int kN = 64;
constexpr int kThreads = 256;            // 8 warps: TMEM lane quadrant = warp & 3, column half = warp >> 2
constexpr int kCols = 32;                // columns of the row component owned by one thread
constexpr int kXtStride = 68;            // floats per transpose-buffer row (conflict-free float4 rows)
constexpr uint32_t kTmemCols = 256;      // A0 [0,64) | A1 [64,128) | A2 [128,192) | D [192,256)
constexpr uint32_t kColA0 = 0, kColA1 = 64, kColA2 = 128, kColD = 192;
constexpr uint32_t kLBO = 128;           // B operand: K-direction core-matrix stride (bytes)
constexpr uint32_t kSBO = 2048;          // B operand: N-direction 8-row-group stride (bytes)
constexpr uint32_t kBopBytes = 16384;    // 64 (N) x 128 (K) fp16
constexpr float kRowFloor = 8.f;         // smallest row bound used for q_B (scaled units)
// thread (r, h): TMEM lane r of the 128-row block [Xr; Xi], columns [kCols h, kCols h + kCols)
static_assert(kThreads == 2 * 128 && 2 * kCols == kN, "two column halves of 32 over 128 lanes");
static_assert(kColA1 == kColA0 + kN && kColA2 == kColA1 + kN && kColD == kColA2 + kN && kColD + kN <= kTmemCols,
              "three A pieces and the accumulator fit the TMEM allocation");
static_assert(kBopBytes == kN * 128 * 2, "B operand: 64 columns x 128 K of fp16");
static_assert(kXtStride >= kN && kXtStride % 4 == 0, "transpose rows hold 64 floats, float4-aligned");

struct __align__(1024) Smem {
  uint8_t bop[2][kBopBytes];             // B0 (fixed point), B1 (residual)
  float xt[128 * kXtStride];             // D transpose buffer, row r = TMEM lane r
  float rlo[kN * 128];                   // compensation of rho, [j][r]
  float smax[2][kThreads];               // per-thread max |B| of the last written stage input
  double red[2][kThreads / 32];
  float redf[kThreads / 32];
  double trp[2];                         // trace partial sums of the two warps owning the diagonal
  double trs[2];                         // partial traces of rho(0) (the same two warps)
  double tr0;                            // trace of the instance's rho(0)
  int eb;                                // the instance's B scale exponent b
  uint64_t mbar;
  uint32_t tmem_base;
};
static_assert(offsetof(Smem, xt) == 2 * kBopBytes && 2 * kBopBytes + sizeof(Smem::xt) >= kN * kN * 16,
              "the B buffers and the transpose buffer, contiguous, hold the staged 64 x 64 complex128 matrix");

struct Args {
  int n, batch, param_batch, n_steps, step0, obs_mode, n_obs, obs_every, obs_per_inst;
  // eb: the B scale exponent b when auto_b is off; sa_half = 2^(a-1); the
  // RK4 constants dt/2, dt, dt/6 (+ its low part) multiplied by 2^-a
  // (accumulator -> B units)
  int eb;
  float sa_half, c_half, c_full, c_sixth, c_sixth_lo;
  double sa_d;
  double trace_tol;
  double2* rho;
  const double2* heff; int64_t heff_stride;
  const double* m_diag; int64_t m_stride;
  const double2* obs_ops; int64_t obs_stride;
  double2* obs_out;
  int32_t* status;
  uint32_t max_wait;
  // drive (kDrive): operators, fp32 pairs [P|1][2][64][64] of Heff and
  // [n_drive][2][64][64] of mu_d (component 0 = re, 1 = im, zero padded),
  // coefficient pairs [n_steps][n_drive] and max_t |c_d|
  int n_drive;
  const double2* drive_ops;
  const float2* heff_pair; int heff_pair_count;
  const float2* drive_pair;
  const float2* coef_pair;
  const double* coef_max;
  // per (matrix, component, row): first and last nonzero column (x > y: none)
  const int2* heff_rng;
  const int2* drive_rng;
  // A operand prepared once per generator (prepare_a_kernel), or null
  const uint4* a_pieces; int64_t a_stride;   // stride in uint4 per parameter set (0: shared)
  int auto_b;                                // per-instance B scale from ||rho(0)||_F
  int n_prefetch;                            // instances per CTA whose inputs are prefetched to L2
  double2* rho_out;                          // final state (may equal rho)
  // extents for the bounds-checked build (elements of rho / rho_out and
  // obs_out, uint4 words of a_pieces)
  size_t rho_elems = kNoExtent, obs_elems = kNoExtent, a_words = kNoExtent;
};

__device__ __forceinline__ double block_sum(double v, double* red, int t) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((t & 31) == 0) red[t >> 5] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int w = 0; w < kThreads / 32; ++w) s += red[w];
  return s;
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
__device__ __forceinline__ uint32_t pack_f2h2(float lo, float hi) {
  const __half2 h = __floats2half2_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// Row quantum from a bound m of |B| on the row (scaled units): |x| <= 1.5 m
// stays within 1023 q for q = 2^(floor(log2(1.5 m)) - 9).  Returns the magic
// constant 1.5 * 2^23 * q: (x + M) - M rounds x to the nearest multiple of q.
__device__ __forceinline__ float row_magic(float m) {
  const int e = ilogbf(fmaxf(1.5f * m, kRowFloor));
  return ldexpf(1.5f, e + 14);
}

// Split 8 consecutive B^T values into b0 (q grid) + b1 (fp16 residual) and store.
__device__ __forceinline__ void store_b8(Smem& S, uint32_t off, const float* x, float magic, float& mx) {
  uint32_t h0[4], h1[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const float u = x[2 * e], w = x[2 * e + 1];
    const float u0 = __fsub_rn(__fadd_rn(u, magic), magic);
    const float w0 = __fsub_rn(__fadd_rn(w, magic), magic);
    h0[e] = pack_f2h2(u0, w0);
    h1[e] = pack_f2h2(__fsub_rn(u, u0), __fsub_rn(w, w0));
    mx = fmaxf(mx, fmaxf(fabsf(u), fabsf(w)));
  }
  *reinterpret_cast<uint4*>(S.bop[0] + off) = make_uint4(h0[0], h0[1], h0[2], h0[3]);
  *reinterpret_cast<uint4*>(S.bop[1] + off) = make_uint4(h1[0], h1[1], h1[2], h1[3]);
}

// x -= c * m on double-float pairs (x = xh + xl, c = ch + cl, m = mh + ml;
// the product to ~46 bits, the difference by an exact two-sum).
__device__ __forceinline__ void df_sub_prod(float& xh, float& xl, float ch, float cl, float mh, float ml) {
  const float ph = __fmul_rn(ch, mh);
  const float pe = __fmaf_rn(ch, mh, -ph);
  const float pl = __fmaf_rn(ch, ml, __fmaf_rn(cl, mh, pe));
  const float sm = __fsub_rn(xh, ph);
  const float bb = __fsub_rn(sm, xh);
  const float er = __fadd_rn(__fsub_rn(xh, __fsub_rn(sm, bb)), __fsub_rn(-ph, bb));
  xh = sm;
  xl = __fadd_rn(__fsub_rn(xl, pl), er);
}

// x = xh + xl (scaled, |x| < 128 q) -> a0 = nearest multiple of q clamped to
// |a0| <= qmax = 127 q (0 for a negligible row) + fp16 residuals a1, a2.
// xh - a0 is exact (both multiples of ulp(xh), difference <= q).
__device__ __forceinline__ void split_a32(float xh, float xl, float magic, float qmax, __half& a0, __half& a1,
                                          __half& a2) {
  float v0 = __fsub_rn(__fadd_rn(xh, magic), magic);
  v0 = fminf(fmaxf(v0, -qmax), qmax);
  const float r = __fadd_rn(__fsub_rn(xh, v0), xl);
  a0 = __float2half_rn(v0);
  a1 = __float2half_rn(r);
  a2 = __float2half_rn(__fsub_rn(r, __half2float(a1)));
}

// Quantum of a block row of A from its bound rmax (scaled units): magic
// rounds to multiples of q = 2^(ilogb(rmax) - 6) and qmax = 127 q clamps
// A0; a row below 2^-18 gets no fixed-point part (magic rounds to integers,
// qmax = 0).
__device__ __forceinline__ void a_row_quantum(float rmax, float& magic, float& qmax) {
  if (rmax >= 0x1p-18f) {
    const int e = ilogbf(rmax);
    magic = ldexpf(1.5f, e - 6 + 23);
    qmax = ldexpf(127.f, e - 6);
  } else {
    magic = 12582912.f;   // 1.5 * 2^23
    qmax = 0.f;
  }
}

// max |A| over the 128 entries of block row (i, component) of 2^a Heff.
__device__ __forceinline__ float a_row_max(const double2* heff, int n, int i, bool xi_row, double sa) {
  float m = 0.f;
#pragma unroll 4
  for (int k = 0; k < 128; ++k) m = fmaxf(m, fabsf((float)(a_elem(heff, n, i, k, xi_row) * sa)));
  return m;
}

// The A pieces of block row (i, component) for k in [64 h + 32 qq, + 32),
// two halves to a word.  Each entry x = 2^a h (exact in FP64) becomes the
// float pair (float) x + (float)(x - (float) x) (~48 bits), split by
// split_a32: three FP64 operations an entry, FP64 being slow on this part.
__device__ __forceinline__ void a_pieces_row(const double2* heff, int n, int i, bool xi_row, int h, int qq, double sa,
                                             float magic, float qmax, uint32_t (&p0)[16], uint32_t (&p1)[16],
                                             uint32_t (&p2)[16]) {
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const int k = 64 * h + 32 * qq + 2 * c;
    __half x0, x1, x2, y0, y1, y2;
    const double u = a_elem(heff, n, i, k, xi_row) * sa;
    const double w = a_elem(heff, n, i, k + 1, xi_row) * sa;
    const float uh = (float)u, wh = (float)w;
    split_a32(uh, (float)(u - (double)uh), magic, qmax, x0, x1, x2);
    split_a32(wh, (float)(w - (double)wh), magic, qmax, y0, y1, y2);
    p0[c] = pack_half2(x0, y0);
    p1[c] = pack_half2(x1, y1);
    p2[c] = pack_half2(x2, y2);
  }
}

// Prepared A operand of one generator: uint4 words in the order
// [piece 3][qq 2][h 2][c4 4][row 128], i.e. the 16 words thread (row, h)
// stores to TMEM columns [32 h + 16 qq, + 16) of piece `piece` are the
// four uint4 at c4 = 0..3, and a warp's 32 rows read 512 contiguous bytes.
constexpr int kAPieceU4 = 3 * 2 * 2 * 4 * 128;    // 98304 bytes per generator
__host__ __device__ __forceinline__ int a_piece_index(int piece, int qq, int h, int c4, int row) {
  return (((piece * 2 + qq) * 2 + h) * 4 + c4) * 128 + row;
}

// Position of element (i, j) of the 64 x 64 double2 matrix staged in shared
// memory: rows of 64, columns XOR-permuted within aligned groups of 8 by
// i & 7, so that a warp's 32 rows at one column (the per-thread component
// reads and writes) spread over 8 bank groups, while 8 consecutive columns
// of a row (the coalesced copies) stay one contiguous 128-byte run.
__device__ __forceinline__ int stage_index(int i, int j) { return i * kN + (j ^ (i & 7)); }

// 2^ea a_elem(...) with the power-of-two scaling as an exponent-field add
// (fpconv::scale_pow2; zeros keep their sign), bit-identical to the FP64
// product.
__device__ __forceinline__ double a_elem_scaled(const double2* heff, int n, int i, int k, bool xi_row, int ea) {
  const double x = a_elem(heff, n, i, k, xi_row);
  return (fpconv::bits64(x) << 1) == 0 ? x : fpconv::scale_pow2(x, ea);
}

// a_row_max and a_pieces_row without the FP64 pipe: the scaling by
// 2^ea = sa through a_elem_scaled and the float pair (float) x,
// (float)(x - (float) x) through fpconv::split_f64, both bit-identical to
// the FP64 instructions, so the pieces are those of the kernel's own split.
// For the stand-alone preparation kernel, whose time is otherwise the FP64
// pipe's (a few operations per clock per SM on this part).
__device__ __forceinline__ float a_row_max_int(const double2* heff, int n, int i, bool xi_row, int ea) {
  float m = 0.f;
#pragma unroll 4
  for (int k = 0; k < 128; ++k) {
    float hi, lo;
    fpconv::split_f64(a_elem_scaled(heff, n, i, k, xi_row, ea), hi, lo);
    m = fmaxf(m, fabsf(hi));
  }
  return m;
}

__device__ __forceinline__ void a_pieces_row_int(const double2* heff, int n, int i, bool xi_row, int h, int qq,
                                                 int ea, float magic, float qmax, uint32_t (&p0)[16],
                                                 uint32_t (&p1)[16], uint32_t (&p2)[16]) {
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const int k = 64 * h + 32 * qq + 2 * c;
    __half x0, x1, x2, y0, y1, y2;
    float uh, ul, wh, wl;
    fpconv::split_f64(a_elem_scaled(heff, n, i, k, xi_row, ea), uh, ul);
    fpconv::split_f64(a_elem_scaled(heff, n, i, k + 1, xi_row, ea), wh, wl);
    split_a32(uh, ul, magic, qmax, x0, x1, x2);
    split_a32(wh, wl, magic, qmax, y0, y1, y2);
    p0[c] = pack_half2(x0, y0);
    p1[c] = pack_half2(x1, y1);
    p2[c] = pack_half2(x2, y2);
  }
}

// The generator staged in shared memory: kN rows of kPrepLd double2, zero
// beyond n.  The padded row puts 8 consecutive rows 16 bytes apart in the
// banks, so a warp's per-thread reads of 32 rows at one column are
// conflict-free.
constexpr int kPrepLd = kN + 1;
constexpr size_t kPrepSmem = (size_t)kN * kPrepLd * sizeof(double2);   // 66,560 bytes

// One CTA per generator, the thread layout of the propagation kernel.
// sa = 2^ea is a normal power of two (|ea| <= 60).  The generator is read
// from global memory once, coalesced, into shared memory; every thread then
// reads its block row there (with stride kPrepLd and every index below
// kN < kPrepLd, a_elem's bound never cuts and the zero fill stands for the
// entries beyond n).
__global__ void __launch_bounds__(kThreads) prepare_a_kernel(const double2* heff, int64_t heff_stride, int n,
                                                              int ea, uint4* out) {
  extern __shared__ double2 hs[];   // [kN][kPrepLd]
  const int t = threadIdx.x, warp = t >> 5;
  const int r = (warp & 3) * 32 + (t & 31), h = warp >> 2;
  const bool xi_row = r >= 64;
  const int i = r & 63;
  const double2* H = heff + (int64_t)blockIdx.x * heff_stride;
  uint4* o = out + (int64_t)blockIdx.x * kAPieceU4;
  for (int e = t; e < kN * kN; e += kThreads) {
    const int ei = e / kN, ej = e % kN;
    hs[ei * kPrepLd + ej] = (ei < n && ej < n) ? H[(int64_t)ei * n + ej] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  float magic, qmax;
  a_row_quantum(a_row_max_int(hs, kPrepLd, i, xi_row, ea), magic, qmax);
#pragma unroll 1
  for (int qq = 0; qq < 2; ++qq) {
    uint32_t p[3][16];
    a_pieces_row_int(hs, kPrepLd, i, xi_row, h, qq, ea, magic, qmax, p[0], p[1], p[2]);
#pragma unroll
    for (int piece = 0; piece < 3; ++piece)
#pragma unroll
      for (int c4 = 0; c4 < 4; ++c4)
        o[a_piece_index(piece, qq, h, c4, r)] =
            make_uint4(p[piece][4 * c4], p[piece][4 * c4 + 1], p[piece][4 * c4 + 2], p[piece][4 * c4 + 3]);
  }
}

// Issue one MMA pass (thread 0) and commit it to mbar; every thread then
// waits on mbar itself (bounded), and the next __syncthreads_or turns any
// thread's timeout into a common abort.  No thread can fall two phases
// behind: each pass is issued only after a barrier that every thread reaches
// after its wait on the previous one.  desc_b0 / desc_b1: descriptors of K
// step 0; K step ks starts 2 * kLBO * ks bytes further, i.e.
// (2 * kLBO / 16) * ks in the descriptor's address field (the operands lie
// far below the field's 256 KB limit, so no carry).
template <bool kExact>
__device__ __forceinline__ void mma_pass(uint32_t tbase, uint64_t desc_b0, uint64_t desc_b1, uint64_t* mbar) {
  constexpr uint32_t idesc = tc::idesc_f16(128, 64, 0);
  constexpr uint64_t kDescStep = 2 * kLBO / 16;
  tc::tc_fence_after();
#pragma unroll
  for (int ks = 0; ks < 8; ++ks) {
    const uint64_t d0 = desc_b0 + kDescStep * ks;
    const uint32_t acc = ks > 0 ? 1u : 0u;
    if (kExact) {
      tc::mma_f16_ts(tbase + kColD, tbase + kColA0 + ks * 8, d0, idesc, acc);
    } else {
      const uint64_t d1 = desc_b1 + kDescStep * ks;
      tc::mma_f16_ts(tbase + kColD, tbase + kColA1 + ks * 8, d0, idesc, acc);
      tc::mma_f16_ts(tbase + kColD, tbase + kColA0 + ks * 8, d1, idesc, 1u);
      tc::mma_f16_ts(tbase + kColD, tbase + kColA1 + ks * 8, d1, idesc, 1u);
      tc::mma_f16_ts(tbase + kColD, tbase + kColA2 + ks * 8, d0, idesc, 1u);
    }
  }
  tc::mma_commit(mbar);
}

template <bool kDrive>
__global__ void __launch_bounds__(kThreads, 2) lindblad_rk4_split_kernel(Args a) {
  extern __shared__ uint8_t smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int t = threadIdx.x, warp = t >> 5;
  const int lq = warp & 3;                  // TMEM lane quadrant
  const int h = warp >> 2;                  // column half
  const int r = lq * 32 + (t & 31);         // row of [Xr; Xi] = TMEM lane (t = 128 h + r)
  const bool is_re = r >= 64;               // rows 64..127 hold Xi and give Re f
  const int i = r & 63;
  const int j0 = kCols * h;
  const bool diag_owner = is_re && (i >> 5) == h;   // holds the (real) diagonal element rho_ii
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
  const uint32_t lane_addr = tbase + ((uint32_t)(lq * 32) << 16);
  const uint64_t desc_b0 = tc::smem_desc_noswizzle(tc::smem_u32(S.bop[0]), kLBO, kSBO);
  const uint64_t desc_b1 = tc::smem_desc_noswizzle(tc::smem_u32(S.bop[1]), kLBO, kSBO);
  const uint32_t brow = (uint32_t)(i >> 3) * kSBO + (uint32_t)(i & 7) * 16u;
  const uint32_t bchunk0 = (is_re ? 0u : 8u) + 4u * (uint32_t)h;
  const float tsign = is_re ? 1.f : -1.f;      // u = own +- transposed element
  float* xrow = S.xt + r * kXtStride;
  const float* xcol = S.xt + (is_re ? 64 : 0) * kXtStride + i;   // X[j][i] at xcol[j * stride]
  uint32_t phase = 0;
  int flags = 0;
  bool aborted = false;
  int g = 0;   // stage counter (parity selects the smax buffer)

  for (int b = blockIdx.x; b < a.batch && !aborted; b += gridDim.x) {
    const int p = b % a.param_batch;
    const double2* heff = a.heff + p * a.heff_stride;
    const float mi = (a.m_diag && i < n) ? (float)a.m_diag[p * a.m_stride + i] : 0.f;

    // inputs of this CTA's next instance into L2 while this one runs
    if (t == 0 && b + (int)gridDim.x < a.batch) {
      const int bn = b + (int)gridDim.x;
      tc::bulk_prefetch_l2(a.rho + (int64_t)bn * n * n, (uint32_t)(n * n * 16));
      if (!kDrive && a.a_pieces && a.a_stride) {
        const uint4* an = a.a_pieces + (int64_t)(bn % a.param_batch) * a.a_stride;
        tc::bulk_prefetch_l2(an, kAPieceU4 * 8u);
        tc::bulk_prefetch_l2(an + kAPieceU4 / 2, kAPieceU4 * 8u);
      }
    }

    // ---- driven: the row's quantum from its bound over the whole drive; the
    // A pieces are written at the start of every step ----
    float magic_a = 0.f, qmax_a = 0.f;
    if (kDrive) {
      double rmax = 0.0;
      for (int k = 0; k < 128; ++k) rmax = fmax(rmax, fabs(a_elem(heff, n, i, k, is_re)));
      for (int dd = 0; dd < a.n_drive; ++dd) {
        double mr = 0.0;
        for (int k = 0; k < 128; ++k) mr = fmax(mr, fabs(a_elem(a.drive_ops + (int64_t)dd * n * n, n, i, k, is_re)));
        rmax += a.coef_max[dd] * mr;
      }
      a_row_quantum((float)(rmax * a.sa_d), magic_a, qmax_a);
    }
    // ---- A operand: block row r of 2^a Heff -> TMEM as A0 + A1 + A2 (this
    // thread: k in [64h, 64h+64)), from the prepared pieces or split here ----
    if (!kDrive) {
      float magic = 0.f, qmax = 0.f;
      if (!a.a_pieces) a_row_quantum(a_row_max(heff, n, i, is_re, a.sa_d), magic, qmax);
      if (a.a_pieces) {
        // all 24 loads in flight before the tensor-memory stores
        const uint4* src = a.a_pieces + (int64_t)p * a.a_stride;
        uint4 v[3][2][4];
#pragma unroll
        for (int piece = 0; piece < 3; ++piece)
#pragma unroll
          for (int qq = 0; qq < 2; ++qq)
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {
              const size_t w = (size_t)p * a.a_stride + a_piece_index(piece, qq, h, c4, r);
              v[piece][qq][c4] = in_bounds(w * 16, 16, a.a_words * 16, a.status) ? src[a_piece_index(piece, qq, h, c4, r)]
                                                                                   : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
        for (int piece = 0; piece < 3; ++piece)
#pragma unroll
          for (int qq = 0; qq < 2; ++qq) {
            uint32_t w[16];
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4) {
              w[4 * c4] = v[piece][qq][c4].x;
              w[4 * c4 + 1] = v[piece][qq][c4].y;
              w[4 * c4 + 2] = v[piece][qq][c4].z;
              w[4 * c4 + 3] = v[piece][qq][c4].w;
            }
            tc::tmem_st16(lane_addr + kColA0 + 64u * piece + 32 * h + 16 * qq, w);
          }
      } else {
#pragma unroll 1
        for (int qq = 0; qq < 2; ++qq) {
          uint32_t p0[16], p1[16], p2[16];
          a_pieces_row(heff, n, i, is_re, h, qq, a.sa_d, magic, qmax, p0, p1, p2);
          const uint32_t col = 32 * h + 16 * qq;
          tc::tmem_st16(lane_addr + kColA0 + col, p0);
          tc::tmem_st16(lane_addr + kColA1 + col, p1);
          tc::tmem_st16(lane_addr + kColA2 + col, p2);
        }
      }
      tc::tmem_wait_st();
    }

    // ---- state: rho(0) is staged through shared memory (the idle B operand
    // and transpose buffers, 64 KB) as a 64 x 64 double2 matrix, loaded with
    // coalesced 16-byte loads; each thread then reads its row component
    // (columns [j0, j0+32)) and, for the Hermiticity check, the transposed
    // element.  Element (i, j) sits at stage_index(i, j).
    double2* stg = reinterpret_cast<double2*>(S.bop[0]);
    {
      const double2* r0 = a.rho + (int64_t)b * n * n;
#pragma unroll 4
      for (int e = t; e < kN * kN; e += kThreads) {
        const int ii = e >> 6, jj = e & 63;
        double2 z = make_double2(0.0, 0.0);
        if (ii < n && jj < n &&
            in_bounds(((size_t)b * n * n + ii * n + jj) * 16, 16, a.rho_elems * 16, a.status))
          z = r0[ii * n + jj];
        stg[stage_index(ii, jj)] = z;
      }
    }
    __syncthreads();
    float rho[kCols], acc[kCols];
    double dtr = 0.0;
    float fro = 0.f;
    bool herm = true;   // rho_ji = conj rho_ij, compared bit for bit (+0 == -0)
    {
      const double* sd = reinterpret_cast<const double*>(stg);
      const int comp = is_re ? 0 : 1;
      const uint64_t flip = is_re ? 0ull : 0x8000000000000000ull;
#pragma unroll
      for (int jj = 0; jj < kCols; ++jj) {
        const int j = j0 + jj;
        const double v = sd[2 * stage_index(i, j) + comp];
        const uint64_t bv = fpconv::bits64(v);
        const uint64_t bw = fpconv::bits64(sd[2 * stage_index(j, i) + comp]) ^ flip;
        herm &= (bv == bw) || ((bv | bw) << 1) == 0;
        float hv, lv;
        fpconv::split_f64(v, hv, lv);   // (float) v and (float)(v - hv) without FP64 instructions
        rho[jj] = hv;
        acc[jj] = 0.f;
        S.rlo[j * 128 + r] = lv;
        fro = __fmaf_rn(hv, hv, fro);
        if (diag_owner && j == i) dtr = v;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
    if (warp == 2 || warp == 7) {   // the warps that own the diagonal
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) dtr += __shfl_xor_sync(0xffffffffu, dtr, o);
      if ((t & 31) == 0) S.trs[warp == 7 ? 1 : 0] = dtr;
    }
    if ((t & 31) == 0) S.redf[warp] = fro;
    __syncthreads();   // (also: every read of the staged matrix is done)
    float fro_all = 0.f;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) fro_all += S.redf[w];
    // B scale: 2^b sqrt(n) ||rho||_F <= 2^13 (sqrt(n) ||rho||_F bounds every
    // |rho_ij(t)|: the trace norm contracts), per instance when auto_b
    int eb = a.eb;
    if (a.auto_b) {
      const float bound = sqrtf((float)n * fro_all);
      eb = 0;
      if (bound > 0.f && isfinite(bound)) {
        const int e = ilogbf(bound);
        eb = (bound == ldexpf(1.f, e)) ? 13 - e : 12 - e;
        eb = max(-60, min(60, eb));
      }
    }
    const float sbi = ldexpf(1.f, eb);
    const float bsign = is_re ? sbi : -sbi;   // natural -> B units of this thread's component
    float mx = 0.f;
    float rho_d = 0.f, acc_d = 0.f, rs_d = 0.f;   // diagonal element (diag_owner only)
#pragma unroll
    for (int jj = 0; jj < kCols; ++jj) {
      const int j = j0 + jj;
      rho[jj] *= bsign;
      S.rlo[j * 128 + r] *= bsign;
      mx = fmaxf(mx, fabsf(rho[jj]));
      if (diag_owner && j == i) rho_d = rho[jj];
    }
    if (!herm) flags |= LIME_FLAG_NOT_HERMITIAN;
    rs_d = rho_d;
    S.smax[g & 1][t] = mx;
    if (t == 0) {   // read after the barriers below (kept out of the step loop's registers)
      S.tr0 = S.trs[0] + S.trs[1];
      S.eb = eb;
    }
    __syncthreads();   // publishes smax
    {
      const float m4 = fmaxf(fmaxf(S.smax[g & 1][i], S.smax[g & 1][64 + i]),
                             fmaxf(S.smax[g & 1][128 + i], S.smax[g & 1][192 + i]));
      const float magic = row_magic(m4);
      float dummy = 0.f;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = rho[8 * c + e];
        store_b8(S, brow + (bchunk0 + c) * kLBO, x, magic, dummy);
      }
    }
    bool tr_pending = false;   // a trace recorded after the last step awaits its check

#pragma unroll 1
    for (int step = 0; step < a.n_steps; ++step) {
      if (kDrive) {
        // A(t) = 2^a (Heff - sum_d c_d(t) mu_d) for this step (the previous
        // step's MMAs, the last readers of TMEM A, have completed: every
        // thread waited on them)
        const int comp = is_re ? (h ? 0 : 1) : (h ? 1 : 0);   // Xr rows [Hr, -Hi], Xi rows [Hi, Hr]
        const float ssa = ((!is_re && h) ? -1.f : 1.f) * (float)a.sa_d;
        const int pp = a.heff_pair_count > 1 ? p : 0;
        const float2* hrow = a.heff_pair + ((size_t)(pp * 2 + comp) * 64 + i) * 64;
        const int2 hr = a.heff_rng[(pp * 2 + comp) * 64 + i];
        const float2* cst = a.coef_pair + (size_t)(a.step0 + step) * a.n_drive;
#pragma unroll 1
        for (int qq = 0; qq < 2; ++qq) {
          uint32_t p0[16], p1[16], p2[16];
#pragma unroll
          for (int c = 0; c < 16; ++c) {
            const int kk = qq * 32 + 2 * c;
            // entries outside a row's nonzero range are zero: not loaded
            float x0h = 0.f, x0l = 0.f, x1h = 0.f, x1l = 0.f;
            if (kk + 1 >= hr.x && kk <= hr.y) {
              const float4 hv = *reinterpret_cast<const float4*>(hrow + kk);
              x0h = hv.x; x0l = hv.y; x1h = hv.z; x1l = hv.w;
            }
            for (int dd = 0; dd < a.n_drive; ++dd) {
              const int2 mr = a.drive_rng[(dd * 2 + comp) * 64 + i];
              if (kk + 1 >= mr.x && kk <= mr.y) {
                const float2 cd = cst[dd];
                const float4 mv =
                    *reinterpret_cast<const float4*>(a.drive_pair + ((size_t)(dd * 2 + comp) * 64 + i) * 64 + kk);
                df_sub_prod(x0h, x0l, cd.x, cd.y, mv.x, mv.y);
                df_sub_prod(x1h, x1l, cd.x, cd.y, mv.z, mv.w);
              }
            }
            __half u0, u1, u2, w0, w1, w2;
            split_a32(x0h * ssa, x0l * ssa, magic_a, qmax_a, u0, u1, u2);
            split_a32(x1h * ssa, x1l * ssa, magic_a, qmax_a, w0, w1, w2);
            p0[c] = pack_half2(u0, w0);
            p1[c] = pack_half2(u1, w1);
            p2[c] = pack_half2(u2, w2);
          }
          const uint32_t col = 32 * h + 16 * qq;
          tc::tmem_st16(lane_addr + kColA0 + col, p0);
          tc::tmem_st16(lane_addr + kColA1 + col, p1);
          tc::tmem_st16(lane_addr + kColA2 + col, p2);
        }
        tc::tmem_wait_st();
      }
#pragma unroll 1
      for (int s = 0; s < 4; ++s, ++g) {
        // ---- pass 1: small products into D ----
        tc::fence_proxy_async_smem();
        tc::tc_fence_before();
        __syncthreads();
        if (t == 0) mma_pass<false>(tbase, desc_b0, desc_b1, &S.mbar);
        if (tr_pending) {
          if (t == 0 && fabs(S.trp[0] + S.trp[1] - S.tr0) > a.trace_tol * fmax(1.0, fabs(S.tr0)))
            flags |= LIME_FLAG_TRACE_DRIFT;
          tr_pending = false;
        }
        int timed_out = tc::mbar_wait_bounded(&S.mbar, phase, a.max_wait) ? 0 : 1;
        phase ^= 1u;
        tc::tc_fence_after();
        float v1[32];   // held in registers across pass 2
        tc::tmem_ld32(lane_addr + kColD + j0, v1);
        // ---- pass 2: the exact product A0.B0 into D ----
        tc::tc_fence_before();
        if (__syncthreads_or(timed_out)) {
          aborted = true;
          break;
        }
        if (t == 0) mma_pass<true>(tbase, desc_b0, desc_b1, &S.mbar);
        timed_out = tc::mbar_wait_bounded(&S.mbar, phase, a.max_wait) ? 0 : 1;
        phase ^= 1u;
        tc::tc_fence_after();
        {
          float v[32];
          tc::tmem_ld32(lane_addr + kColD + j0, v);
#pragma unroll
          for (int e = 0; e < 8; ++e)
            *reinterpret_cast<float4*>(xrow + j0 + 4 * e) =
                make_float4(__fadd_rn(v[4 * e], v1[4 * e]), __fadd_rn(v[4 * e + 1], v1[4 * e + 1]),
                            __fadd_rn(v[4 * e + 2], v1[4 * e + 2]), __fadd_rn(v[4 * e + 3], v1[4 * e + 3]));
        }
        // dephasing jump term m_i rho_ii folded into the diagonal of X (it
        // enters Re f_ii = X_ii + X_ii twice, hence the half; rs_d is in B units)
        if (diag_owner) xrow[i] = __fmaf_rn(mi * a.sa_half, rs_d, xrow[i]);
        const float m4 = fmaxf(fmaxf(S.smax[g & 1][i], S.smax[g & 1][64 + i]),
                               fmaxf(S.smax[g & 1][128 + i], S.smax[g & 1][192 + i]));
        const float magic = row_magic(m4);
        if (__syncthreads_or(timed_out)) {
          aborted = true;
          break;
        }

        // RK4 in accumulator units: u = 2^(a+b) (+-f), acc += w u, next stage
        // input R + c u (c = dt/2 or dt in B units); the last stage combines
        // R + (acc + u) dt/6 on the (hi, lo) pair and clears acc.
        float nmx = 0.f;
        if (s < 3) {
          const float cst = (s == 2) ? a.c_full : a.c_half;
          const float wgt = (s == 0) ? 1.f : 2.f;
          float rs_d_next = rs_d;
          if (diag_owner) {
            const float xd = xrow[i];
            const float ud = __fadd_rn(xd, xd);
            acc_d = __fmaf_rn(wgt, ud, acc_d);
            rs_d_next = __fmaf_rn(cst, ud, rho_d);
          }
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            float own[16];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const float4 o = *reinterpret_cast<const float4*>(xrow + j0 + q * 16 + 4 * e);
              own[4 * e] = o.x; own[4 * e + 1] = o.y; own[4 * e + 2] = o.z; own[4 * e + 3] = o.w;
            }
            float nxt[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) {
              const int jj = q * 16 + e;
              const float u = __fmaf_rn(tsign, xcol[(j0 + jj) * kXtStride], own[e]);
              acc[jj] = __fmaf_rn(wgt, u, acc[jj]);
              nxt[e] = __fmaf_rn(cst, u, rho[jj]);
            }
#pragma unroll
            for (int h8 = 0; h8 < 2; ++h8)
              store_b8(S, brow + (bchunk0 + 2 * q + h8) * kLBO, nxt + 8 * h8, magic, nmx);
          }
          rs_d = rs_d_next;
        } else {
          if (diag_owner) {
            const float xd = xrow[i];
            float lo_d = S.rlo[i * 128 + r];
            rho_d = rk4_final_f32(rho_d, acc_d, __fadd_rn(xd, xd), a.c_sixth, a.c_sixth_lo, lo_d);
            acc_d = 0.f;
            rs_d = rho_d;
          }
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            float own[16];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const float4 o = *reinterpret_cast<const float4*>(xrow + j0 + q * 16 + 4 * e);
              own[4 * e] = o.x; own[4 * e + 1] = o.y; own[4 * e + 2] = o.z; own[4 * e + 3] = o.w;
            }
#pragma unroll
            for (int e = 0; e < 16; ++e) {
              const int jj = q * 16 + e;
              const float u = __fmaf_rn(tsign, xcol[(j0 + jj) * kXtStride], own[e]);
              float lo = S.rlo[(j0 + jj) * 128 + r];
              rho[jj] = rk4_final_f32(rho[jj], acc[jj], u, a.c_sixth, a.c_sixth_lo, lo);
              S.rlo[(j0 + jj) * 128 + r] = lo;
              acc[jj] = 0.f;
            }
#pragma unroll
            for (int h8 = 0; h8 < 2; ++h8)
              store_b8(S, brow + (bchunk0 + 2 * q + h8) * kLBO, rho + q * 16 + 8 * h8, magic, nmx);
          }
        }
        S.smax[(g + 1) & 1][t] = nmx;
      }
      if (aborted) break;

      // ---- observables / trace after the step ----
      const int gstep = a.step0 + step;
      if (((gstep + 1) % a.obs_every) == 0) {
        const int slot = (gstep + 1) / a.obs_every - 1;
        double2* orow = a.obs_out + ((int64_t)b * a.obs_per_inst + slot) * a.n_obs;
        const size_t obase = ((size_t)b * a.obs_per_inst + slot) * a.n_obs;
        const double dval =
            diag_owner ? fpconv::scale_pow2(fpconv::widen_f32(rho_d) + fpconv::widen_f32(S.rlo[i * 128 + r]), -S.eb)
                       : 0.0;
        if (a.obs_mode == 1) {
          if (diag_owner && i < a.n_obs && in_bounds((obase + i) * 16, 16, a.obs_elems * 16, a.status))
            orow[i] = make_double2(dval, 0.0);
        } else if (a.obs_mode == 2) {
          const double2* E0 = a.obs_ops + p * a.obs_stride;
          for (int o = 0; o < a.n_obs; ++o) {
            const double2* E = E0 + (int64_t)o * n * n;
            float pr = 0.f, pi = 0.f;
            if (i < n) {
#pragma unroll
              for (int jj = 0; jj < kCols; ++jj) {
                const int j = j0 + jj;
                if (j < n) {
                  const double2 ev = E[(int64_t)j * n + i];   // E[j][i]
                  const float er = (float)ev.x, ei = (float)ev.y;
                  // B units: rho[jj] = 2^b Re rho_ij, or -2^b Im rho_ij
                  if (is_re) {
                    pr = __fmaf_rn(er, rho[jj], pr);
                    pi = __fmaf_rn(ei, rho[jj], pi);
                  } else {
                    pr = __fmaf_rn(ei, rho[jj], pr);
                    pi = __fmaf_rn(-er, rho[jj], pi);
                  }
                }
              }
            }
            const double sr = fpconv::scale_pow2(block_sum((double)pr, S.red[0], t), -S.eb);
            const double si = fpconv::scale_pow2(block_sum((double)pi, S.red[1], t), -S.eb);
            if (t == 0 && in_bounds((obase + o) * 16, 16, a.obs_elems * 16, a.status)) orow[o] = make_double2(sr, si);
          }
        }
        if (a.trace_tol > 0.0) {
          // the diagonal lives in warps 2 (i < 32) and 7 (i >= 32); their sums
          // are compared with tr0 by thread 0 after the next barrier
          if (warp == 2 || warp == 7) {
            double v = (diag_owner && i < n) ? dval : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if ((t & 31) == 0) S.trp[warp == 7 ? 1 : 0] = v;
          }
          tr_pending = true;
        }
      }
    }
    if (aborted) break;

    // ---- final state: hi + lo of every element into the staged matrix
    // (one FP64 addition each; widening, power-of-two scale and sign without
    // FP64 instructions), then coalesced 16-byte stores ----
    __syncthreads();   // the last stage's reads of the transpose buffer are done
    {
      double* sd = reinterpret_cast<double*>(stg);
      const int comp = is_re ? 0 : 1;
      const int ebi = -S.eb;
      const uint64_t neg = is_re ? 0ull : 0x8000000000000000ull;   // B units hold -2^b Im rho
#pragma unroll
      for (int jj = 0; jj < kCols; ++jj) {
        const int j = j0 + jj;
        const double v = fpconv::scale_pow2(fpconv::widen_f32(rho[jj]) + fpconv::widen_f32(S.rlo[j * 128 + r]), ebi);
        if (!isfinite(rho[jj])) flags |= LIME_FLAG_NONFINITE;
        sd[2 * stage_index(i, j) + comp] = fpconv::from_bits64(fpconv::bits64(v) ^ neg);
      }
    }
    __syncthreads();
    {
      double2* out = a.rho_out + (int64_t)b * n * n;
#pragma unroll 4
      for (int e = t; e < n * n; e += kThreads) {
        const int ii = e / n, jj = e - ii * n;
        if (in_bounds(((size_t)b * n * n + e) * 16, 16, a.rho_elems * 16, a.status)) out[e] = stg[stage_index(ii, jj)];
      }
    }
    __syncthreads();   // smax / rlo of this instance are no longer read
    if (tr_pending && t == 0 && fabs(S.trp[0] + S.trp[1] - S.tr0) > a.trace_tol * fmax(1.0, fabs(S.tr0)))
      flags |= LIME_FLAG_TRACE_DRIFT;
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

// ---------------------------------------------------------------- drive preparation
// Workspace of a driven call: fp32 hi/lo pairs of Heff ([P|1][2][64][64]),
// of the drive operators ([n_drive][2][64][64]) and of the coefficients
// ([n_steps][n_drive]), max_t |c_d| ([n_drive] doubles), and the nonzero
// column range of every row of the pair arrays ([P|1][2][64] and
// [n_drive][2][64] int2).
struct DriveWs {
  size_t ops, coef, cmax, hrng, drng, total;
};
static DriveWs drive_ws(int P, int n_drive, int n_steps) {
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  DriveWs w;
  w.ops = al((size_t)P * 2 * 4096 * sizeof(float2));
  w.coef = w.ops + al((size_t)n_drive * 2 * 4096 * sizeof(float2));
  w.cmax = w.coef + al((size_t)n_steps * n_drive * sizeof(float2));
  w.hrng = w.cmax + al((size_t)n_drive * sizeof(double));
  w.drng = w.hrng + al((size_t)P * 2 * 64 * sizeof(int2));
  w.total = w.drng + al((size_t)n_drive * 2 * 64 * sizeof(int2));
  return w;
}

// one thread per row of a [count][2][64][64] pair array: its first and last
// nonzero column ((64, -1) for an all-zero row)
__global__ void range_kernel(const float2* pairs, int rows, int2* rng) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const float2* row = pairs + (size_t)r * 64;
  int lo = 64, hi = -1;
  for (int j = 0; j < 64; ++j) {
    const float2 v = row[j];
    if (v.x != 0.f || v.y != 0.f) {
      lo = min(lo, j);
      hi = j;
    }
  }
  rng[r] = make_int2(lo, hi);
}

// count matrices (n x n, stride elements apart) -> [count][2][64][64] pairs, zero padded
__global__ void pair_kernel(const double2* src, int64_t stride, int count, int n, float2* dst) {
  const int64_t total = (int64_t)count * 4096;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / 4096), ij = (int)(e % 4096), i = ij / 64, j = ij % 64;
    double2 v = make_double2(0.0, 0.0);
    if (i < n && j < n) v = src[c * stride + (int64_t)i * n + j];
    const float rh = (float)v.x, ih = (float)v.y;
    dst[((int64_t)c * 2 + 0) * 4096 + ij] = make_float2(rh, (float)(v.x - (double)rh));
    dst[((int64_t)c * 2 + 1) * 4096 + ij] = make_float2(ih, (float)(v.y - (double)ih));
  }
}

// one block per drive operator: coefficient pairs and max_t |c_d|
__global__ void coef_kernel(const double* coef, int n_steps, int n_drive, float2* cp, double* cmax) {
  __shared__ double red[32];
  const int dd = blockIdx.x;
  double m = 0.0;
  for (int s = threadIdx.x; s < n_steps; s += blockDim.x) {
    const double v = coef[(int64_t)s * n_drive + dd];
    const float hv = (float)v;
    cp[(int64_t)s * n_drive + dd] = make_float2(hv, (float)(v - (double)hv));
    m = fmax(m, fabs(v));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
    cmax[dd] = r;
  }
}

}  // namespace split
}  // namespace lime

using namespace lime;

static int g_num_sms = 0;

extern "C" size_t lime_lindblad_split_workspace(int32_t n, int32_t param_batch, int32_t n_drive, int32_t n_steps) {
  if (n <= 0 || param_batch <= 0 || n_drive < 0 || n_steps < 0) return 0;
  if (n_drive == 0) return 0;
  return split::drive_ws(param_batch, n_drive, n_steps).total;
}

extern "C" size_t lime_lindblad_split_prepared_bytes(int32_t n, int32_t count) {
  if (n <= 0 || n > split::kN || count <= 0) return 0;
  return (size_t)count * split::kAPieceU4 * sizeof(uint4);
}

extern "C" int lime_lindblad_split_prepare(const LimeLindbladSplitPrepareDesc* d, void* stream) {
  if (!d) return LIME_ERR_ARG;
  if (d->n <= 0 || d->count <= 0 || !d->heff || !d->out) return LIME_ERR_ARG;
  if (d->n > split::kN) return LIME_ERR_UNSUPPORTED;
  if (d->heff_stride < 0 || (d->count > 1 && d->heff_stride < (int64_t)d->n * d->n)) return LIME_ERR_ARG;
  if (d->scale_a_log2 < -60 || d->scale_a_log2 > 60) return LIME_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(d->heff) & 15) != 0 || (reinterpret_cast<uintptr_t>(d->out) & 15) != 0)
    return LIME_ERR_ARG;
  if (d->out_bytes < lime_lindblad_split_prepared_bytes(d->n, d->count)) return LIME_ERR_WORKSPACE;
  LIME_CUDA_TRY(cudaFuncSetAttribute(split::prepare_a_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)split::kPrepSmem));
  split::prepare_a_kernel<<<d->count, split::kThreads, split::kPrepSmem, (cudaStream_t)stream>>>(
      reinterpret_cast<const double2*>(d->heff), d->heff_stride, d->n, (int)d->scale_a_log2,
      reinterpret_cast<uint4*>(d->out));
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch();
  return LIME_OK;
}

extern "C" int lime_lindblad_rk4_split(const LimeLindbladSplitDesc* d, void* stream) {
  if (!d) return LIME_ERR_ARG;
  if (d->n <= 0 || d->batch <= 0 || d->n_steps < 0 || d->n_obs < 0 || d->chunk_steps < 0) return LIME_ERR_ARG;
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
  if (d->n_drive < 0) return LIME_ERR_ARG;
  if (d->n_drive > 0) {
    if (!d->drive_ops || !d->drive_coef || !d->workspace) return LIME_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(d->workspace) & 255) != 0) return LIME_ERR_ARG;
    if (d->workspace_bytes < lime_lindblad_split_workspace(d->n, pb, d->n_drive, d->n_steps))
      return LIME_ERR_WORKSPACE;
  }
  if (d->a_pieces) {
    if (d->n_drive > 0) return LIME_ERR_ARG;   // a driven A is split on the device every step
    if ((reinterpret_cast<uintptr_t>(d->a_pieces) & 15) != 0) return LIME_ERR_ARG;
    if (d->a_stride != 0 && d->a_stride != (int64_t)split::kAPieceU4 * 16) return LIME_ERR_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(d->rho) & 15) != 0 || (reinterpret_cast<uintptr_t>(d->heff) & 15) != 0 ||
      (reinterpret_cast<uintptr_t>(d->rho_out) & 15) != 0)
    return LIME_ERR_ARG;
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
  a.eb = d->scale_b_log2;
  a.sa_half = ldexpf(1.f, d->scale_a_log2 - 1);
  {
    // the fp32 constants of the natural-unit update, then scaled by 2^-a (exact)
    const float c6 = (float)(d->dt / 6.0);
    const float c6lo = (float)(d->dt / 6.0 - (double)c6);
    a.c_half = ldexpf((float)(d->dt / 2.0), -d->scale_a_log2);
    a.c_full = ldexpf((float)d->dt, -d->scale_a_log2);
    a.c_sixth = ldexpf(c6, -d->scale_a_log2);
    a.c_sixth_lo = ldexpf(c6lo, -d->scale_a_log2);
  }
  a.trace_tol = d->trace_tol;
  a.rho = reinterpret_cast<double2*>(d->rho);
  a.heff = reinterpret_cast<const double2*>(d->heff); a.heff_stride = d->heff_stride;
  a.m_diag = d->m_diag; a.m_stride = d->m_stride;
  a.obs_ops = reinterpret_cast<const double2*>(d->obs_ops); a.obs_stride = d->obs_stride;
  a.obs_out = reinterpret_cast<double2*>(d->obs_out);
  a.status = d->status;
  a.max_wait = 1u << 26;
  a.a_pieces = reinterpret_cast<const uint4*>(d->a_pieces);
  a.a_stride = d->a_stride / 16;
  a.auto_b = d->auto_scale_b != 0;
  a.rho_out = reinterpret_cast<double2*>(d->rho_out ? d->rho_out : d->rho);
  a.rho_elems = (size_t)d->batch * d->n * d->n;
  a.obs_elems = (size_t)d->batch * a.obs_per_inst * (d->n_obs > 0 ? d->n_obs : 0);
  a.a_words = (size_t)(d->a_stride ? pb : 1) * split::kAPieceU4;
  cudaStream_t st = (cudaStream_t)stream;
  const bool driven = d->n_drive > 0;
  if (driven) {
    const split::DriveWs w = split::drive_ws(pb, d->n_drive, d->n_steps);
    uint8_t* ws = static_cast<uint8_t*>(d->workspace);
    const int hp = d->heff_stride == 0 ? 1 : pb;
    a.n_drive = d->n_drive;
    a.drive_ops = reinterpret_cast<const double2*>(d->drive_ops);
    a.heff_pair = reinterpret_cast<const float2*>(ws);
    a.heff_pair_count = hp;
    a.drive_pair = reinterpret_cast<const float2*>(ws + w.ops);
    a.coef_pair = reinterpret_cast<const float2*>(ws + w.coef);
    a.coef_max = reinterpret_cast<const double*>(ws + w.cmax);
    a.heff_rng = reinterpret_cast<const int2*>(ws + w.hrng);
    a.drive_rng = reinterpret_cast<const int2*>(ws + w.drng);
    split::pair_kernel<<<304, 256, 0, st>>>(a.heff, d->heff_stride, hp, d->n, reinterpret_cast<float2*>(ws));
    LIME_CUDA_TRY(cudaGetLastError());
    split::pair_kernel<<<64, 256, 0, st>>>(a.drive_ops, (int64_t)d->n * d->n, d->n_drive, d->n,
                                           reinterpret_cast<float2*>(ws + w.ops));
    LIME_CUDA_TRY(cudaGetLastError());
    split::coef_kernel<<<d->n_drive, 256, 0, st>>>(d->drive_coef, d->n_steps, d->n_drive,
                                                   reinterpret_cast<float2*>(ws + w.coef),
                                                   reinterpret_cast<double*>(ws + w.cmax));
    LIME_CUDA_TRY(cudaGetLastError());
    split::range_kernel<<<(hp * 128 + 127) / 128, 128, 0, st>>>(a.heff_pair, hp * 128,
                                                                reinterpret_cast<int2*>(ws + w.hrng));
    LIME_CUDA_TRY(cudaGetLastError());
    split::range_kernel<<<(d->n_drive * 128 + 127) / 128, 128, 0, st>>>(a.drive_pair, d->n_drive * 128,
                                                                         reinterpret_cast<int2*>(ws + w.drng));
    LIME_CUDA_TRY(cudaGetLastError());
    count_launch(5);
  }
  const int ctas_per_sm = d->ctas_per_sm > 0 ? d->ctas_per_sm : 2;
  const int grid = (int)((d->batch < ctas_per_sm * g_num_sms) ? d->batch : ctas_per_sm * g_num_sms);
  const size_t smem = sizeof(split::Smem) + 1024;
  auto kern = driven ? split::lindblad_rk4_split_kernel<true> : split::lindblad_rk4_split_kernel<false>;
  LIME_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // bounded launches: about 2^22 instance-steps per launch
  const double per_cta = (double)((d->batch + grid - 1) / grid);
  int chunk = d->chunk_steps > 0 ? d->chunk_steps
                                 : (int)fmax(1.0, fmin((double)d->n_steps, 4194304.0 / (per_cta * grid)));
  if (a.obs_every > 1) chunk = ((chunk + a.obs_every - 1) / a.obs_every) * a.obs_every;
  for (int s0 = 0; s0 < d->n_steps; s0 += chunk) {
    a.step0 = s0;
    a.n_steps = (d->n_steps - s0 < chunk) ? d->n_steps - s0 : chunk;
    kern<<<grid, split::kThreads, smem, st>>>(a);
    LIME_CUDA_TRY(cudaGetLastError());
    count_launch();
    a.rho = a.rho_out;   // the next launch continues from this one's final state
  }
  return LIME_OK;
}
