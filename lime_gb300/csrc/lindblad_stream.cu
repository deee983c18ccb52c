// General Lindblad RK4 on the sm_103a tensor cores: any dimension, dense
// collapse operators, split precision (the streaming tile of
// stream_gemm.cuh).
//
// Generator (lime/oqs.py:706-723, written with Heff = H - i/2 sum L^dag L):
//     f(rho) = -i (X - X^dag) + sum_k L_k rho L_k^dag + M o rho,   X = Heff rho
// per RK4 stage, for every instance, as two GEMMs of the real block form
// [Yr | Yi] = [Ar | Ai] . [[Sr, Si], [-Si, Sr]]:
//   GEMM 1   [X; Y_1; ...; Y_K] = [Heff; L_1; ...; L_K] . rho_s
//            (A constant: converted once; B = the stage input rho_s)
//   GEMM 2   Z = [L_1 | ... | L_K] . [Y_1^dag; ...; Y_K^dag] = sum_k L_k rho_s L_k^dag
//            (A constant; B = Y^dag, written by GEMM 1's epilogue)
// GEMM 2's epilogue assembles f = Z - i(X - X^dag) + M o rho_s (X from
// GEMM 1, transposed reads through L2) and runs the RK4 stage update; with
// no dense operator a plain kernel does the same without Z.  rho_s is
// Hermitian (a non-Hermitian start runs as its two Hermitian parts), which
// is what makes rho_s X^dag-free and Z = Z^dag.
//
// Layouts per instance (n padded to np, a multiple of 64; W = 2 np): state
// hi, lo, RK4 accumulator, X and the stage input fp32 planar [W][np] with
// element [comp * np + x][y] = comp-part of rho[y][x]; operands pre-tiled
// in 16 KB pieces (piece_off).

#include "stream_gemm.cuh"

namespace lime {
namespace lsm {

using sg::kBM;
using sg::kBN;
using sg::kFStride;
using sg::kPiece;

struct Args {
  int n, np, W, NT, K, P, G;          // G = generator sets (1 = shared)
  int KC1, KC2, MT1, MT2;
  float sb, inv_sb, sy, inv_sy;
  sg::RK4 rk;
  const uint8_t* A1[3];               // [G][MT1][KC1] pieces
  const uint8_t* A2[3];               // [G][MT2][KC2] pieces
  const float* rinv1;                 // [G][MT1 * 128]
  const float* rinv2;                 // [G][MT2 * 128]
  const uint8_t* B1c[2];              // [B][NT][KC1] current stage input
  uint8_t* B1n[2];                    // next stage input
  uint8_t* B2[2];                     // [B][NT][KC2]  Y^dag
  float* Xg;                          // [B][W][np]
  const float* Sc;                    // [B][W][np] current stage input (M term)
  float* Sn;                          // next stage input
  float* Phi;                         // [B][W][np]
  float* Plo;
  float* Acc;
  const double2* m;                   // [P|1][n][n] or null
  int64_t m_stride;
  const double* mdg;                  // diagonal M (real, [P|1][n]) instead of m, or null
  int64_t mdg_stride;
  bool keep_s;                        // maintain the fp32 stage-input copy (Sc / Sn)
  const int* sb_exp_dev;              // GEMM 1: B scale exponent read from the device (or null: inv_sb)
  float* stage_store;                 // finish_kernel: also store the stage input here ([B][W][np]) or null
  int32_t* status;
  uint32_t max_wait;
  // buffer extents for the bounds-checked build: bytes of one A1 / A2 piece
  // set and of one B1 / B2 piece buffer, floats of one [B][W][np] state array
  size_t a1_bytes = kNoExtent, a2_bytes = kNoExtent, b1_bytes = kNoExtent, b2_bytes = kNoExtent;
  size_t st_floats = kNoExtent;
  // GEMM 2 over the upper tiles of the Hermitian Z only (np a multiple of
  // 128 with two or more row tiles): a strictly upper tile also stores its
  // raw Z into Zg ([B][W][np], the layout of Xg), and zlower_kernel updates
  // the elements of the lower tiles from Z[y][x] = conj(Z[x][y])
  int zhalf = 0;
  float* Zg = nullptr;
};

// GEMM 2 tiles per instance: all MT2 x NT, or with zhalf the upper ones,
// (row tile mt, column block xb) with mt <= xb for each of the two
// components
__host__ __device__ __forceinline__ int gemm2_tiles(const Args& a) {
  const int xbs = a.np / 128;
  return a.zhalf ? xbs * (xbs + 1) : a.MT2 * a.NT;
}

__device__ __forceinline__ size_t inst_floats(const Args& a) { return (size_t)a.W * a.np; }

// f for 8 rows y..y+7 of state column jj of instance b: Z (or 0) + the X
// terms + the M term, in place.  tr: the transposed X run the X terms need,
// X_c[x][y..y+7] with c = Im for a real column and Re for an imaginary one.
__device__ __forceinline__ void assemble_f_tr(const Args& a, int b, int jj, int y, const float (&tr)[8],
                                              float (&f)[8]) {
  const int np = a.np;
  const bool im = jj >= np;
  const int x = im ? jj - np : jj;
  const float* X = a.Xg + (size_t)b * inst_floats(a);
  float u[8];
  if (!im) {
    // Re f = Xi[y][x] + Xi[x][y]
    sg::ld8(X + (size_t)(np + x) * np + y, u);
#pragma unroll
    for (int i = 0; i < 8; ++i) f[i] = __fadd_rn(f[i], __fadd_rn(u[i], tr[i]));
  } else {
    // Im f = Xr[x][y] - Xr[y][x]
    sg::ld8(X + (size_t)x * np + y, u);
#pragma unroll
    for (int i = 0; i < 8; ++i) f[i] = __fadd_rn(f[i], __fsub_rn(tr[i], u[i]));
  }
  if (a.mdg != nullptr) {
    // diagonal M: only (M o rho)_xx = M_xx rho_xx, real (the stage input's
    // diagonal is real), so only the real column x meets it, in row x
    if (!im && x < a.n && x >= y && x < y + 8) {
      const double* Md = a.mdg + (a.mdg_stride ? (int64_t)(b % a.P) * a.mdg_stride : 0);
      const float sxx = a.Sc[(size_t)b * inst_floats(a) + (size_t)x * np + x];
      const float mr = (float)Md[x];
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (y + i == x) f[i] = __fmaf_rn(mr, sxx, f[i]);
    }
  } else if (a.m != nullptr && x < a.n) {
    const double2* M = a.m + (a.m_stride ? (int64_t)(b % a.P) * a.m_stride : 0);
    const float* S = a.Sc + (size_t)b * inst_floats(a);
    float sr[8], si[8];
    sg::ld8(S + (size_t)x * np + y, sr);
    sg::ld8(S + (size_t)(np + x) * np + y, si);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (y + i < a.n) {
        const double2 mv = M[(size_t)(y + i) * a.n + x];
        const float mr = (float)mv.x, mi = (float)mv.y;
        f[i] = im ? __fmaf_rn(mr, si[i], __fmaf_rn(mi, sr[i], f[i]))
                  : __fmaf_rn(mr, sr[i], __fmaf_rn(-mi, si[i], f[i]));
      }
    }
  }
}

// The same with the transposed run read from global memory (strided).
__device__ __forceinline__ void assemble_f(const Args& a, int b, int jj, int y, float (&f)[8]) {
  const int np = a.np;
  const bool im = jj >= np;
  const int x = im ? jj - np : jj;
  const float* X = a.Xg + (size_t)b * inst_floats(a) + (size_t)(im ? 0 : np) * np;
  float tr[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) tr[i] = X[(size_t)(y + i) * np + x];
  assemble_f_tr(a, b, jj, y, tr, f);
}

// RK4 stage update of 8 state rows and the next stage input (B1 pieces and,
// for the M term, the fp32 copy).
__device__ __forceinline__ void update8(const Args& a, int b, int jj, int y, const float (&f)[8], bool& bad,
                                        bool& range) {
  const size_t base = (size_t)b * inst_floats(a);
  if (!in_bounds((base + (size_t)jj * a.np + y) * sizeof(float), 8 * sizeof(float), a.st_floats * sizeof(float),
                 a.status))
    return;
  float sv[8];
  sg::rk4_stage8(a.rk, a.Phi + base, a.Plo + base, a.Acc + base, (size_t)jj * a.np + y, f, sv, bad);
  if (a.keep_s) sg::st8(a.Sn + base + (size_t)jj * a.np + y, sv);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    sv[i] = __fmul_rn(sv[i], a.sb);
    range |= !(fabsf(sv[i]) <= sg::kBMax);
  }
  const bool im = jj >= a.np;
  const size_t boff = (size_t)b * a.NT * a.KC1 * kPiece;
  sg::scatter_cplx8(a.B1n[0] + boff, a.B1n[1] + boff, a.KC1, a.np, a.np, y, im ? jj - a.np : jj, im, sv,
                    a.b1_bytes - boff, a.status);
}

// The fused epilogue of tile (b, mt, nt), run by the kEpiThreads epilogue
// threads: kZ = false: GEMM 1 (X rows into Xg, Y_k rows as Y^dag into
// GEMM 2's B operand); kZ = true: GEMM 2, f and the RK4 stage update.  The
// finished tile is read through park1(col, row) (one value) and
// park8(col, row, v) (rows row..row+7).
template <bool kZ, class P1, class P8>
__device__ __forceinline__ void fused_epilogue(const Args& a, int b, int mt, int nt, const P1& park1,
                                               const P8& park8) {
  const int t = threadIdx.x, lane = t & 31;
  const int u = t - sg::kEpiFirst, ew = u >> 5;
  const int np = a.np;
  bool bad = false, range = false;
  if (!kZ) {
    // ---- X rows (block 0): the tile columns into Xg, runs of 8 rows
    const int nlo = lane & 7, glo = lane >> 3;
#pragma unroll 1
    for (int wi = ew; wi < 64; wi += sg::kEpiWarps) {
      const int jl = (wi >> 2) * 8 + nlo;
      const int dl = ((wi & 3) * 4 + glo) * 8;
      const int R = mt * kBM + dl;
      const size_t xo = (size_t)b * inst_floats(a) + (size_t)(nt * kBN + jl) * np + R;
      if (R < np && in_bounds(xo * sizeof(float), 8 * sizeof(float), a.st_floats * sizeof(float), a.status)) {
        float v[8];
        park8(jl, dl, v);
        sg::st8(a.Xg + xo, v);
      }
    }
    // ---- Y_k rows (blocks 1..K): Y^dag into B2, runs of 8 columns of one row
    const int r = u & 127, o0 = u >> 7;
    constexpr int kGroups = sg::kEpiThreads / 128;
    const int R = mt * kBM + r;
    const int blk = R / np, yrow = R - blk * np;
    if (blk >= 1 && blk <= a.K) {
      uint8_t* B20 = a.B2[0] + (size_t)b * a.NT * a.KC2 * kPiece;
      uint8_t* B21 = a.B2[1] + (size_t)b * a.NT * a.KC2 * kPiece;
#pragma unroll 1
      for (int i = 0; i < 16 / kGroups; ++i) {
        const int cl = 8 * (o0 + kGroups * i);
        const int jj = nt * kBN + cl;
        const bool im = jj >= np;
        const int x = im ? jj - np : jj;
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          // S2[(k-1) np + x][yrow] = conj(Y_k[yrow][x]): real part Yr, imaginary part -Yi
          const float y = park1(cl + e, r);
          v[e] = __fmul_rn(im ? -y : y, a.sy);
          range |= !(fabsf(v[e]) <= sg::kBMax);
        }
        sg::scatter_cplx8(B20, B21, a.KC2, a.K * np, np, (blk - 1) * np + x, yrow, im, v,
                          a.b2_bytes - (size_t)b * a.NT * a.KC2 * kPiece, a.status);
      }
    }
  } else {
    // ---- f = Z + X terms + M term and the RK4 stage update, runs of 8 rows
    const int nlo = lane & 7, glo = lane >> 3;
#pragma unroll 1
    for (int wi = ew; wi < 64; wi += sg::kEpiWarps) {
      const int jl = (wi >> 2) * 8 + nlo;
      const int dl = ((wi & 3) * 4 + glo) * 8;
      const int y = mt * kBM + dl, jj = nt * kBN + jl;
      if (y < np) {
        float f[8];
        park8(jl, dl, f);
        if (a.zhalf && mt < (nt * kBN % np) / 128) {
          // raw Z of a strictly upper tile, for the transposed lower one
          const size_t zo = (size_t)b * inst_floats(a) + (size_t)jj * np + y;
          if (in_bounds(zo * sizeof(float), 8 * sizeof(float), a.st_floats * sizeof(float), a.status))
            sg::st8(a.Zg + zo, f);
        }
        assemble_f(a, b, jj, y, f);
        update8(a, b, jj, y, f, bad, range);
      }
    }
  }
  if (bad) atomicOr(a.status, LIME_FLAG_NONFINITE);
  if (range) atomicOr(a.status, LIME_FLAG_RANGE);
}

// Tile `local` of a GEMM 1 (kZ = false) or GEMM 2 launch over a.batch
// instances: its operands and position.
template <bool kZ>
__device__ __forceinline__ void gemm_tile_of(const Args& a, int local, sg::Tile& T, int& b, int& mt, int& nt) {
  const int MT = kZ ? a.MT2 : a.MT1;
  const int KC = kZ ? a.KC2 : a.KC1;
  const int per = kZ ? gemm2_tiles(a) : MT * a.NT;
  b = local / per;
  const int tile = local % per;
  if (kZ && a.zhalf) {
    // upper tiles of component comp: column block xb holds row tiles 0..xb
    const int xbs = a.np / 128, half = xbs * (xbs + 1) / 2;
    const int comp = tile / half;
    int u = tile - comp * half, xb = 0;
    while (u > xb) {
      u -= xb + 1;
      ++xb;
    }
    mt = u;
    nt = comp * xbs + xb;
  } else {
    mt = tile / a.NT;
    nt = tile % a.NT;
  }
  const int g = a.G == 1 ? 0 : b % a.P;
  const size_t aoff = ((size_t)g * MT + mt) * KC * kPiece;
  const size_t boff = ((size_t)b * a.NT + nt) * KC * kPiece;
  for (int i = 0; i < 3; ++i) T.A[i] = (kZ ? a.A2[i] : a.A1[i]) + aoff;
  for (int i = 0; i < 2; ++i) T.B[i] = (kZ ? a.B2[i] : a.B1c[i]) + boff;
  T.c0 = 0;
  T.n_chunks = KC;
  T.row_inv = (kZ ? a.rinv2 : a.rinv1) + ((size_t)g * MT + mt) * kBM;
  T.inv_sb = kZ ? a.inv_sy : (a.sb_exp_dev != nullptr ? ldexpf(1.f, -*a.sb_exp_dev) : a.inv_sb);
  T.max_wait = a.max_wait;
  T.a_avail = (kZ ? a.a2_bytes : a.a1_bytes) - aoff;
  T.b_avail = (kZ ? a.b2_bytes : a.b1_bytes) - boff;
  T.status = a.status;
}

// kZ = false: GEMM 1 (X and Y_k rows); kZ = true: GEMM 2 and the stage update.
// One tile per CTA.
template <bool kZ>
__global__ void __launch_bounds__(sg::kThreads, 1) gemm_kernel(Args a) {
  extern __shared__ uint8_t smem_raw[];
  sg::Smem& S = *reinterpret_cast<sg::Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  sg::setup(S);
  sg::Tile T;
  int b, mt, nt;
  gemm_tile_of<kZ>(a, blockIdx.x, T, b, mt, nt);
  const float* ft = S.tile();
  if (sg::mainloop(S, T) && !*(volatile int*)&S.abort) {
    fused_epilogue<kZ>(
        a, b, mt, nt, [&](int c, int r) { return ft[c * kFStride + r]; },
        [&](int c, int r, float (&v)[8]) { sg::ld8(ft + c * kFStride + r, v); });
  }
  sg::teardown(S, a.status);
}

// The GEMM 1 or GEMM 2 tiles of several instance groups (different
// dimensions and operator counts) in one persistent launch: CTA j runs
// tiles j, j + gridDim.x, ... of the concatenated tile list, whose groups
// the host orders by decreasing chunks per tile (largest tiles first).
constexpr int kMaxGroups = 16;
struct Groups {
  int n_groups, n_items;
  int start[kMaxGroups + 1];          // first tile of each group in the list
  Args g[kMaxGroups];
};
static_assert(sizeof(Groups) <= 30000, "kernel parameter space");

template <bool kZ>
__global__ void __launch_bounds__(sg::kThreads, 1) gemm_groups_kernel(const __grid_constant__ Groups m) {
  extern __shared__ uint8_t smem_raw[];
  sg::Smem& S = *reinterpret_cast<sg::Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  sg::setup(S);
  sg::Seq q;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  auto group_of = [&](int item) {
    int gi = 0;
    while (gi + 1 < m.n_groups && item >= m.start[gi + 1]) ++gi;
    return gi;
  };
  if (warp < 2) {
    if (lane == 0) {
      bool alive = true;
      for (int item = blockIdx.x; item < m.n_items && alive; item += gridDim.x) {
        const int gi = group_of(item);
        sg::Tile T;
        int b, mt, nt;
        gemm_tile_of<kZ>(m.g[gi], item - m.start[gi], T, b, mt, nt);
        alive = warp == 0 ? sg::seq_produce(S, T, q) : sg::seq_mma(S, T, q);
      }
      if (warp == 0)
        sg::seq_produce_end(S, q, m.g[0].max_wait);
      else
        sg::seq_mma_end(S, m.g[0].max_wait);
    }
  } else {
    const float* ft = S.lo;
    for (int item = blockIdx.x; item < m.n_items; item += gridDim.x) {
      const int gi = group_of(item);
      sg::Tile T;
      int b, mt, nt;
      gemm_tile_of<kZ>(m.g[gi], item - m.start[gi], T, b, mt, nt);
      const bool ok = sg::seq_drain(S, T, q);
      const bool stop = sg::epi_bar_or(!ok || *(volatile int*)&S.abort);
      if (!stop) {
        fused_epilogue<kZ>(
            m.g[gi], b, mt, nt, [&](int c, int r) { return ft[sg::park_idx(c, r)]; },
            [&](int c, int r, float (&v)[8]) { sg::ld8_park(ft, c, r, v); });
      }
      sg::epi_bar();   // the parked tile is read before the next drain clears it
      if (stop) break;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (t == 0 && S.abort)
    for (int i = 0; i < m.n_groups; ++i) atomicOr(m.g[i].status, LIME_FLAG_TIMEOUT);
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(S.tmem_base, sg::kTmemCols);
  }
}

// 32 x 32 tiles of the state for the elementwise stage kernels: the
// transposed X runs come through shared memory (coalesced loads), the rest
// is read in place.  Block (instance, x tile, y tile); thread -> (component,
// column x, run of 8 rows).
struct TileItem {
  int b, jj, y;
  float tr[8];
};

__device__ __forceinline__ TileItem load_tile_item(const Args& a, float (*T)[32][33]) {
  const int np = a.np, tiles = np / 32;
  const int b = blockIdx.x / (tiles * tiles);
  const int t2 = blockIdx.x % (tiles * tiles);
  const int x0 = (t2 / tiles) * 32, y0 = (t2 % tiles) * 32;
  const float* X = a.Xg + (size_t)b * inst_floats(a);
  // T[c][yy][xx] = X_c[x0 + xx][y0 + yy]  (row x0 + xx, column y0 + yy)
  for (int idx = threadIdx.x; idx < 2 * 32 * 32; idx += blockDim.x) {
    const int c = idx >> 10, yy = (idx >> 5) & 31, xx = idx & 31;
    T[c][yy][xx] = X[(size_t)(c * np + y0 + yy) * np + x0 + xx];
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int comp = t >> 7, xl = (t >> 2) & 31, yl = (t & 3) * 8;
  TileItem it;
  it.b = b;
  it.jj = comp * np + x0 + xl;
  it.y = y0 + yl;
#pragma unroll
  for (int i = 0; i < 8; ++i) it.tr[i] = T[comp ? 0 : 1][yl + i][xl];
  return it;
}

// The stage update without dense operators (no GEMM 2).
__global__ void __launch_bounds__(256) finish_kernel(Args a) {
  __shared__ float T[2][32][33];
  const TileItem it = load_tile_item(a, T);
  bool bad = false, range = false;
  if (a.stage_store != nullptr) {
    const size_t e = (size_t)it.b * inst_floats(a) + (size_t)it.jj * a.np + it.y;
    float sc[8];
    sg::ld8(a.Sc + e, sc);
    sg::st8(a.stage_store + e, sc);
  }
  float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  assemble_f_tr(a, it.b, it.jj, it.y, it.tr, f);
  update8(a, it.b, it.jj, it.y, f, bad, range);
  if (bad) atomicOr(a.status, LIME_FLAG_NONFINITE);
  if (range) atomicOr(a.status, LIME_FLAG_RANGE);
}

// The stage update of the lower tiles of Z (row tile above the column
// block) when GEMM 2 ran over the upper ones only: Z[y][x] = conj(Z[x][y])
// from the strictly upper tiles' raw Z in Zg, then f and the RK4 update as
// in GEMM 2's epilogue.  One thread per run of 8 rows of one state column.
__global__ void __launch_bounds__(256) zlower_kernel(Args a, int batch) {
  const int np = a.np, xbs = np / 128;
  const int pairs = xbs * (xbs - 1) / 2;               // (mt, xb) with mt > xb
  const size_t per_inst = (size_t)2 * pairs * 128 * 16;  // components x pairs x columns x 8-row runs
  const size_t total = (size_t)batch * per_inst;
  bool bad = false, range = false;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(q / per_inst);
    size_t r = q % per_inst;
    const int run = (int)(r % 16);
    r /= 16;
    const int xl = (int)(r % 128);
    r /= 128;
    int u = (int)(r % pairs);
    const int comp = (int)(r / pairs);
    int mt = 1;   // lower pair u: row tile mt, column block xb < mt
    while (u >= mt) {
      u -= mt;
      ++mt;
    }
    const int xb = u;
    const int x = xb * 128 + xl, y = mt * 128 + run * 8;
    const int jj = comp * np + x;
    const float* Z = a.Zg + (size_t)b * inst_floats(a);
    float f[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      // Re Z[y][x] = Re Z[x][y];  Im Z[y][x] = -Im Z[x][y]  (Zg[c np + x'][y'] = Z_c[y'][x'])
      const float v = Z[(size_t)(comp * np + y + i) * np + x];
      f[i] = comp ? -v : v;
    }
    assemble_f(a, b, jj, y, f);
    update8(a, b, jj, y, f, bad, range);
  }
  if (bad) atomicOr(a.status, LIME_FLAG_NONFINITE);
  if (range) atomicOr(a.status, LIME_FLAG_RANGE);
}

// A pieces: GEMM 1 rows (R = blk np + y: Heff for blk 0, L_blk otherwise)
// and GEMM 2 rows (y: [L_1 | ... | L_K] row y).  One block per row.
struct ConvertOut {
  uint8_t* A1[3];                     // [G][MT1][KC1] pieces
  uint8_t* A2[3];                     // [G][MT2][KC2] pieces
  float* rinv1;                       // [G][MT1 * 128]
  float* rinv2;                       // [G][MT2 * 128]
};

// only_heff: convert just the Heff rows (block 0) of GEMM 1, np per set
// (the driven generator re-splits Heff(t) every step).
__global__ void convert_kernel(const double2* heff, int64_t heff_stride, const double2* l_ops, int64_t l_stride,
                               Args a, ConvertOut out, int only_heff) {
  const int rows1 = a.MT1 * kBM, rows2 = a.MT2 * kBM;
  const int per_g = only_heff ? a.np : rows1 + (a.K > 0 ? rows2 : 0);
  const int g = blockIdx.x / per_g;
  const int q = blockIdx.x % per_g;
  const int n = a.n, np = a.np;
  if (q < rows1) {
    const int R = q, blk = R / np, y = R - blk * np;
    const bool valid = blk <= a.K && y < n;
    const double2* src = blk == 0 ? heff + (heff_stride ? (int64_t)g * heff_stride : 0)
                                  : l_ops + (l_stride ? (int64_t)g * l_stride : 0) + (int64_t)(blk - 1) * n * n;
    auto elem = [&](int kk) -> double2 {
      return kk < n ? src[(int64_t)y * n + kk] : make_double2(0.0, 0.0);
    };
    const size_t go = (size_t)g * a.MT1 * a.KC1 * kPiece;
    sg::convert_row(elem, R, valid, np, np, a.KC1, out.A1[0] + go, out.A1[1] + go, out.A1[2] + go,
                    out.rinv1 + (size_t)g * rows1);
  } else {
    const int y = q - rows1;
    const double2* src = l_ops + (l_stride ? (int64_t)g * l_stride : 0);
    auto elem = [&](int kk) -> double2 {
      const int k = kk / np, x = kk - k * np;
      return x < n ? src[(int64_t)k * n * n + (int64_t)y * n + x] : make_double2(0.0, 0.0);
    };
    const size_t go = (size_t)g * a.MT2 * a.KC2 * kPiece;
    sg::convert_row(elem, y, y < n, a.K * np, a.K * np, a.KC2, out.A2[0] + go, out.A2[1] + go, out.A2[2] + go,
                    out.rinv2 + (size_t)g * rows2);
  }
}

// Heff(t) = Heff - sum_q c_q H_q for every generator set (the driven
// generator, lime/oqs.py:1716-1722), FP64.
__global__ void heff_t_kernel(const double2* heff, int64_t heff_stride, int G, int n, const double2* ops,
                              const double* coef, int n_drive, double2* out) {
  const size_t nn = (size_t)n * n;
  const size_t total = (size_t)G * nn;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
    const size_t g = q / nn, e = q % nn;
    double2 v = heff[(heff_stride ? g * heff_stride : 0) + e];
    for (int k = 0; k < n_drive; ++k) {
      const double2 h = ops[(size_t)k * nn + e];
      v.x -= coef[k] * h.x;
      v.y -= coef[k] * h.y;
    }
    out[q] = v;
  }
}

// state, stage-input copy and first B1 from rho0 [B][n][n]
__global__ void init_kernel(Args a, const double2* rho, int batch) {
  const size_t runs = (size_t)a.W * (a.np / 8);
  const size_t total = (size_t)batch * runs;
  bool range = false;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(q / runs);
    const int rem = (int)(q % runs);
    const int jj = rem / (a.np / 8), y = (rem % (a.np / 8)) * 8;
    const bool im = jj >= a.np;
    const int x = im ? jj - a.np : jj;
    float hv[8], lv[8], sv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      double v = 0.0;
      if (x < a.n && y + i < a.n) {
        const double2 z = rho[((size_t)b * a.n + y + i) * a.n + x];
        v = im ? z.y : z.x;
      }
      hv[i] = (float)v;
      lv[i] = (float)(v - (double)hv[i]);
      sv[i] = __fmul_rn(hv[i], a.sb);
      range |= !(fabsf(sv[i]) <= sg::kBMax);
    }
    const size_t e = (size_t)b * inst_floats(a) + (size_t)jj * a.np + y;
    sg::st8(a.Phi + e, hv);
    sg::st8(a.Plo + e, lv);
    if (a.keep_s) sg::st8(a.Sn + e, hv);
    const size_t boff = (size_t)b * a.NT * a.KC1 * kPiece;
    sg::scatter_cplx8(a.B1n[0] + boff, a.B1n[1] + boff, a.KC1, a.np, a.np, y, x, im, sv);
  }
  if (range) atomicOr(a.status, LIME_FLAG_RANGE);
}

// obs[b][slot][o] = Tr(E_o rho_b) = sum_xy E_o[x][y] rho[y][x], fp64 from hi + lo;
// diag: E holds only the diagonals E_o[x][x] ([P|1][n_obs][n]), n terms
__global__ void observe_kernel(Args a, const double2* E, int64_t e_stride, int n_obs, double2* out, int n_slots,
                               int slot, int diag) {
  const int b = blockIdx.x / n_obs, o = blockIdx.x % n_obs;
  const int per = diag ? a.n : a.n * a.n;
  const double2* Eo = E + (e_stride ? (int64_t)(b % a.P) * e_stride : 0) + (int64_t)o * per;
  const size_t base = (size_t)b * inst_floats(a);
  double sr = 0.0, si = 0.0;
  for (int q = threadIdx.x; q < per; q += blockDim.x) {
    const int x = diag ? q : q / a.n, y = diag ? q : q - x * a.n;
    const double2 ev = Eo[q];
    // a zero entry adds exactly zero (projectors and dipoles are sparse);
    // non-finite states are flagged by the stage kernels
    if (ev.x == 0.0 && ev.y == 0.0) continue;
    const size_t er = base + (size_t)x * a.np + y, ei = base + (size_t)(a.np + x) * a.np + y;
    const double pr = (double)a.Phi[er] + (double)a.Plo[er];
    const double pi = (double)a.Phi[ei] + (double)a.Plo[ei];
    sr += ev.x * pr - ev.y * pi;
    si += ev.x * pi + ev.y * pr;
  }
  __shared__ double red[32];
  sr = block_sum<128>(sr, red);
  si = block_sum<128>(si, red);
  if (threadIdx.x == 0) out[((size_t)b * n_slots + slot) * n_obs + o] = make_double2(sr, si);
}

__global__ void final_kernel(Args a, double2* rho, int batch) {
  const size_t total = (size_t)batch * a.n * a.n;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(q / ((size_t)a.n * a.n));
    const int rem = (int)(q % ((size_t)a.n * a.n));
    const int y = rem / a.n, x = rem - y * a.n;
    const size_t base = (size_t)b * inst_floats(a);
    const size_t er = base + (size_t)x * a.np + y, ei = base + (size_t)(a.np + x) * a.np + y;
    rho[q] = make_double2((double)a.Phi[er] + (double)a.Plo[er], (double)a.Phi[ei] + (double)a.Plo[ei]);
  }
}

// ---------------------------------------------------------------- discrete adjoint
// Backward pass of the RK4 steps above (the FP64 adjoint kernel's recursion,
// lime_lindblad_adjoint_f64): per step, with lam the adjoint state after the
// step and ab_i the inputs of the adjoint generator L^dag(x) = -i(G x -
// x G^dag) + conj(M) o x (G = -Heff^dag, run through the same GEMM 1 and
// assemble_f with the adjoint operands):
//   ab_4 = dt/6 lam;           yb_4 = L^dag ab_4
//   ab_3 = dt/3 lam + dt yb_4;  ab_2 = dt/3 lam + dt/2 yb_3;  ab_1 = dt/6 lam + dt/2 yb_2
//   lam <- lam + yb_4 + yb_3 + yb_2 + yb_1
// and the parameter gradients pair ab_i with the forward stage input y_i.
struct AdjState {
  float* Lhi;        // [B][W][np] adjoint state (fp32 pair, compensated)
  float* Llo;
  float* LAcc;       // sum of the yb of the current step
  unsigned* lmax;    // device: max |lam| of the current step (float bits)
  int* sl_exp;       // device: exponent of the adjoint B scale for the current step
  float bound;       // |ab| <= bound * max |lam| (dt/2: ab_i = c lam + c' yb)
};

// Per step, the adjoint stage inputs are scaled by the power of two that puts
// bound * max |lam| at 2^13 / 1.25 (lam changes by orders of magnitude over a
// backward pass, one scale for all steps would waste the fixed-point range).
__global__ void adj_scale_kernel(AdjState j) {
  const float m = __uint_as_float(*j.lmax) * j.bound;
  int e = 0;
  if (m > 0.f && isfinite(m)) {
    e = (int)floorf(log2f(6553.6f / m));
    e = e < -60 ? -60 : (e > 60 ? 60 : e);
  }
  *j.sl_exp = e;
  *j.lmax = 0u;
}

// Source of the observables recorded after this step, lam += Herm(g E^dag)
// (torch's convention dL = Re sum conj(g) d obs), and max |lam| of the step.
// Observable sources into the adjoint state: (g conj(E_ji) + conj(g) E_ij) / 2
// per element (torch's convention dL = Re sum conj(g) d obs), formed in FP64
// from E, or, with Q (obs_coef), as Re g Q.x + Im g Q.y from its fp32
// coefficient pairs ([P|1][n_obs][component][x][row], two FMAs an element).
__global__ void adj_source_kernel(Args a, AdjState j, int batch, const double2* E, int64_t e_stride, int n_obs,
                                  const double2* gsrc, int n_slots, int slot, const float2* Q) {
  const size_t runs = (size_t)a.W * (a.np / 8);
  const size_t total = (size_t)batch * runs;
  float mx = 0.f;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(q / runs);
    const int rem = (int)(q % runs);
    const int jj = rem / (a.np / 8), y = (rem % (a.np / 8)) * 8;
    const bool im = jj >= a.np;
    const int x = im ? jj - a.np : jj;
    const size_t e = (size_t)b * inst_floats(a) + (size_t)jj * a.np + y;
    float hi[8];
    sg::ld8(j.Lhi + e, hi);
    if (slot >= 0 && x < a.n && Q != nullptr) {
      float lo[8];
      sg::ld8(j.Llo + e, lo);
      const float2* Qb = Q + (e_stride ? (int64_t)(b % a.P) * n_obs * 2 * a.n * a.n : 0);
      const double2* g = gsrc + ((size_t)b * n_slots + slot) * n_obs;
      float src[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      for (int o = 0; o < n_obs; ++o) {
        const float gx = (float)g[o].x, gy = (float)g[o].y;
        const float2* Qo = Qb + (((size_t)o * 2 + (im ? 1 : 0)) * a.n + x) * a.n + y;
#pragma unroll
        for (int i = 0; i < 8; ++i)
          if (y + i < a.n) {
            const float2 q = Qo[i];
            src[i] = __fmaf_rn(gx, q.x, __fmaf_rn(gy, q.y, src[i]));
          }
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (y + i < a.n) hi[i] = rk4_final_f32(hi[i], 0.f, src[i], 1.f, 0.f, lo[i]);
      sg::st8(j.Lhi + e, hi);
      sg::st8(j.Llo + e, lo);
    } else if (slot >= 0 && x < a.n) {
      float lo[8];
      sg::ld8(j.Llo + e, lo);
      const double2* Eb = E + (e_stride ? (int64_t)(b % a.P) * e_stride : 0);
      const double2* g = gsrc + ((size_t)b * n_slots + slot) * n_obs;
#pragma unroll 1
      for (int i = 0; i < 8; ++i) {
        const int row = y + i;
        if (row >= a.n) break;
        double sr = 0.0, si = 0.0;
        for (int o = 0; o < n_obs; ++o) {
          const double2* Eo = Eb + (int64_t)o * a.n * a.n;
          const double2 eji = Eo[(size_t)x * a.n + row], eij = Eo[(size_t)row * a.n + x], gv = g[o];
          // (g conj(E_ji) + conj(g) E_ij) / 2
          sr += 0.5 * ((gv.x * eji.x + gv.y * eji.y) + (gv.x * eij.x + gv.y * eij.y));
          si += 0.5 * ((gv.y * eji.x - gv.x * eji.y) + (gv.x * eij.y - gv.y * eij.x));
        }
        const float src = (float)(im ? si : sr);
        hi[i] = rk4_final_f32(hi[i], 0.f, src, 1.f, 0.f, lo[i]);
      }
      sg::st8(j.Lhi + e, hi);
      sg::st8(j.Llo + e, lo);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) mx = fmaxf(mx, fabsf(hi[i]));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(j.lmax, __float_as_uint(mx));
}

// ab_4 = dt/6 lam as the next GEMM 1 input (fp32 copy and scaled B pieces).
__global__ void adj_start_kernel(Args a, AdjState j, int batch, float dt6) {
  const size_t runs = (size_t)a.W * (a.np / 8);
  const size_t total = (size_t)batch * runs;
  const float sl = ldexpf(1.f, *j.sl_exp);
  bool range = false;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(q / runs);
    const int rem = (int)(q % runs);
    const int jj = rem / (a.np / 8), y = (rem % (a.np / 8)) * 8;
    const bool im = jj >= a.np;
    const int x = im ? jj - a.np : jj;
    const size_t e = (size_t)b * inst_floats(a) + (size_t)jj * a.np + y;
    float ab[8];
    sg::ld8(j.Lhi + e, ab);
#pragma unroll
    for (int i = 0; i < 8; ++i) ab[i] = __fmul_rn(dt6, ab[i]);
    sg::st8(a.Sn + e, ab);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      ab[i] = __fmul_rn(ab[i], sl);
      range |= !(fabsf(ab[i]) <= sg::kBMax);
    }
    const size_t boff = (size_t)b * a.NT * a.KC1 * kPiece;
    sg::scatter_cplx8(a.B1n[0] + boff, a.B1n[1] + boff, a.KC1, a.np, a.np, y, x, im, ab);
  }
  if (range) atomicOr(a.status, LIME_FLAG_RANGE);
}

// yb_i = L^dag ab_i (Xg = G ab_i from GEMM 1, ab_i in Sc) and the next
// adjoint stage input (stage i = 4, 3, 2) or the new lam (i = 1).
__global__ void __launch_bounds__(256) adj_finish_kernel(Args a, AdjState j, int stage_i, float c_l, float c_y) {
  __shared__ float T[2][32][33];
  const TileItem it = load_tile_item(a, T);
  const float sl = ldexpf(1.f, *j.sl_exp);
  bool range = false;
  const int b = it.b, jj = it.jj, y = it.y;
  const bool im = jj >= a.np;
  const size_t e = (size_t)b * inst_floats(a) + (size_t)jj * a.np + y;
  float f[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  assemble_f_tr(a, b, jj, y, it.tr, f);
  float acc[8], hi[8];
  if (stage_i == 4) {
    sg::st8(j.LAcc + e, f);
  } else {
    sg::ld8(j.LAcc + e, acc);
    if (stage_i > 1) {
#pragma unroll
      for (int i = 0; i < 8; ++i) acc[i] = __fadd_rn(acc[i], f[i]);
      sg::st8(j.LAcc + e, acc);
    } else {
      float lo[8];
      sg::ld8(j.Lhi + e, hi);
      sg::ld8(j.Llo + e, lo);
#pragma unroll
      for (int i = 0; i < 8; ++i) hi[i] = rk4_final_f32(hi[i], acc[i], f[i], 1.f, 0.f, lo[i]);
      sg::st8(j.Lhi + e, hi);
      sg::st8(j.Llo + e, lo);
    }
  }
  if (stage_i > 1) {
    float nx[8];
    sg::ld8(j.Lhi + e, hi);
#pragma unroll
    for (int i = 0; i < 8; ++i) nx[i] = __fmaf_rn(c_l, hi[i], __fmul_rn(c_y, f[i]));
    sg::st8(a.Sn + e, nx);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      nx[i] = __fmul_rn(nx[i], sl);
      range |= !(fabsf(nx[i]) <= sg::kBMax);
    }
    const size_t boff = (size_t)b * a.NT * a.KC1 * kPiece;
    sg::scatter_cplx8(a.B1n[0] + boff, a.B1n[1] + boff, a.KC1, a.np, a.np, y, im ? jj - a.np : jj, im, nx);
  }
  if (range) atomicOr(a.status, LIME_FLAG_RANGE);
}

// Gradient contributions of one stage for the chain model (site energies on
// the diagonal, nearest-neighbour bonds, site dephasing rates), pairing the
// adjoint stage input ab with the forward stage input y (both Hermitian):
//   d/dH_kk   += 2 sum_x Im(conj(ab_kx) y_kx)
//   d/dJ_k    += 2 sum_x Im(conj(ab_kx) y_k+1,x) + Im(conj(ab_k+1,x) y_kx)
//   d/dgamma_k -= sum_{x != k} Re(conj(ab_kx) y_kx)
// One block per (instance, run of 8 rows), threads over the columns.
__global__ void adj_grad_kernel(Args a, const float* ab, const float* yst, int batch, double* gd, double* gb,
                                double* gg) {
  const int runs = a.np / 8;
  const int b = blockIdx.x / runs, k0 = (blockIdx.x % runs) * 8;
  if (b >= batch || k0 >= a.n) return;
  const int n = a.n, np = a.np;
  const float* A = ab + (size_t)b * inst_floats(a);
  const float* Y = yst + (size_t)b * inst_floats(a);
  // per-thread partial sums in fp32 (a thread sees a few columns; fp64
  // arithmetic runs at a small fraction of the fp32 rate on this part), the
  // block reduction in fp64
  float pf[24];
#pragma unroll
  for (int i = 0; i < 24; ++i) pf[i] = 0.f;
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    float ar[9], ai[9], yr[9], yi[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      const int k = k0 + i;
      const bool ok = k < np;
      ar[i] = ok ? A[(size_t)x * np + k] : 0.f;
      ai[i] = ok ? A[(size_t)(np + x) * np + k] : 0.f;
      yr[i] = ok ? Y[(size_t)x * np + k] : 0.f;
      yi[i] = ok ? Y[(size_t)(np + x) * np + k] : 0.f;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int k = k0 + i;
      if (k < n) {
        pf[i] = __fmaf_rn(2.f, __fmaf_rn(ar[i], yi[i], -ai[i] * yr[i]), pf[i]);
        if (x != k) pf[16 + i] -= __fmaf_rn(ar[i], yr[i], ai[i] * yi[i]);
        if (k + 1 < n)
          pf[8 + i] = __fmaf_rn(2.f, __fmaf_rn(ar[i], yi[i + 1], -ai[i] * yr[i + 1]) +
                                         __fmaf_rn(ar[i + 1], yi[i], -ai[i + 1] * yr[i]), pf[8 + i]);
      }
    }
  }
  double part[24];
#pragma unroll
  for (int i = 0; i < 24; ++i) part[i] = (double)pf[i];
  __shared__ double red[4][24];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < 24; ++i) {
    double v = part[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) red[w][i] = v;
  }
  __syncthreads();
  if (threadIdx.x < 24) {
    const int i = threadIdx.x;
    double v = 0.0;
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww) v += red[ww][i];
    const int k = k0 + (i & 7);
    const int nb = n > 1 ? n - 1 : 1;
    if (k < n) {
      if (i < 8) atomicAdd(gd + (size_t)b * n + k, v);
      else if (i < 16) { if (k + 1 < n) atomicAdd(gb + (size_t)b * nb + k, v); }
      else atomicAdd(gg + (size_t)b * n + k, v);
    }
  }
}

}  // namespace lsm
}  // namespace lime

using namespace lime;

namespace {

struct LsmLayout {
  int np, W, NT, KC1, KC2, MT1, MT2, G;
  int zhalf;                           // GEMM 2 over the upper tiles of Z only
  size_t a1, a2, r1, r2, b1, b2, st;   // bytes of one piece set / array
  size_t total;
};

LsmLayout lsm_layout(int n, int batch, int G, int K) {
  LsmLayout l;
  l.np = (n + 63) / 64 * 64;
  l.W = 2 * l.np;
  l.NT = l.W / 128;
  l.KC1 = 2 * l.np / sg::kCK;
  l.KC2 = 2 * K * l.np / sg::kCK;
  l.MT1 = ((1 + K) * l.np + 127) / 128;
  l.MT2 = K > 0 ? (l.np + 127) / 128 : 0;
  l.G = G;
  l.a1 = (size_t)G * l.MT1 * l.KC1 * sg::kPiece;
  l.a2 = (size_t)G * l.MT2 * l.KC2 * sg::kPiece;
  l.r1 = ((size_t)G * l.MT1 * 128 * sizeof(float) + 1023) / 1024 * 1024;
  l.r2 = ((size_t)G * l.MT2 * 128 * sizeof(float) + 1023) / 1024 * 1024;
  l.b1 = (size_t)batch * l.NT * l.KC1 * sg::kPiece;
  l.b2 = (size_t)batch * l.NT * l.KC2 * sg::kPiece;
  l.st = (size_t)batch * l.W * l.np * sizeof(float);
  l.zhalf = (K > 0 && l.np % 128 == 0 && l.np >= 256) ? 1 : 0;
  // A1 x3, A2 x3, row scales, B1 x2 pieces x2 buffers, B2 x2 pieces,
  // X, stage input x2, Phi, Plo, Acc (+ Z of the upper tiles)
  l.total = 3 * l.a1 + 3 * l.a2 + l.r1 + l.r2 + 4 * l.b1 + 2 * l.b2 + (6 + l.zhalf) * l.st + 4096;
  return l;
}

int lsm_generators(int P, int64_t heff_stride, int K, int64_t l_stride) {
  return (heff_stride == 0 && (K == 0 || l_stride == 0)) ? 1 : P;
}

}  // namespace

extern "C" size_t lime_lindblad_stream_workspace(int32_t n, int32_t batch, int32_t n_generators, int32_t n_ops) {
  if (n <= 0 || batch <= 0 || n_generators <= 0 || n_ops < 0) return 0;
  // (+ one FP64 Heff(t) per generator set for driven generators)
  return lsm_layout(n, batch, n_generators, n_ops).total + (size_t)n_generators * n * n * 16;
}

namespace {

// The buffers of one streaming propagation inside its workspace.
struct LsmRun {
  lsm::Args a;
  lsm::ConvertOut co;
  LsmLayout L;
  uint8_t* B1[2][2];
  float* Sbuf[2];
  double2* heff_t;
  int B, K, G;
};

// Validates d, lays out its workspace, converts the operands and loads the
// initial state (two launches on st).
int lsm_prepare(const LimeLindbladStreamDesc* d, LsmRun& r, cudaStream_t st, int64_t& launches) {
  if (!d || d->n <= 0 || d->batch <= 0 || d->n_ops < 0 || d->n_steps < 0 || d->n_obs < 0) return LIME_ERR_ARG;
  if (!d->rho || !d->heff || !d->workspace || !d->status) return LIME_ERR_ARG;
  if (d->n_ops > 0 && !d->l_ops) return LIME_ERR_ARG;
  if (d->n_obs > 0 && (!d->obs_ops || !d->obs_out)) return LIME_ERR_ARG;
  if (d->heff_stride < 0 || d->l_stride < 0 || d->m_stride < 0 || d->obs_stride < 0) return LIME_ERR_ARG;
  if (d->m_diag_stride < 0 || (d->obs_diag & ~1)) return LIME_ERR_ARG;
  if (d->scale_b_log2 < -60 || d->scale_b_log2 > 60 || d->scale_y_log2 < -60 || d->scale_y_log2 > 60)
    return LIME_ERR_ARG;
  if (d->n > 4096 || d->n_ops > 64) return LIME_ERR_UNSUPPORTED;
  const int P = d->param_batch > 0 ? d->param_batch : d->batch;
  if (P > d->batch) return LIME_ERR_ARG;
  if (!(d->dt == d->dt)) return LIME_ERR_ARG;
  if (d->n_drive < 0 || (d->n_drive > 0 && (!d->drive_ops || !d->drive_coef))) return LIME_ERR_ARG;
  const int K = d->n_ops;
  const int G = lsm_generators(P, d->heff_stride, K, d->l_stride);
  const LsmLayout L = lsm_layout(d->n, d->batch, G, K);
  const size_t drive_bytes = d->n_drive > 0 ? (size_t)G * d->n * d->n * sizeof(double2) : 0;
  if (d->workspace_bytes < L.total + drive_bytes) return LIME_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(d->workspace) & 1023) != 0) return LIME_ERR_ARG;
  r.L = L;
  r.B = d->batch;
  r.K = K;
  r.G = G;

  uint8_t* w = reinterpret_cast<uint8_t*>(d->workspace);
  lsm::Args& a = r.a;
  lsm::ConvertOut& co = r.co;
  a = lsm::Args{};
  co = lsm::ConvertOut{};
  a.n = d->n; a.np = L.np; a.W = L.W; a.NT = L.NT; a.K = K; a.P = P; a.G = G;
  a.KC1 = L.KC1; a.KC2 = L.KC2; a.MT1 = L.MT1; a.MT2 = L.MT2;
  for (int i = 0; i < 3; ++i) { a.A1[i] = co.A1[i] = w; w += L.a1; }
  for (int i = 0; i < 3; ++i) { a.A2[i] = co.A2[i] = w; w += L.a2; }
  a.rinv1 = co.rinv1 = reinterpret_cast<float*>(w); w += L.r1;
  a.rinv2 = co.rinv2 = reinterpret_cast<float*>(w); w += L.r2;
  for (int bb = 0; bb < 2; ++bb)
    for (int i = 0; i < 2; ++i) { r.B1[bb][i] = w; w += L.b1; }
  for (int i = 0; i < 2; ++i) { a.B2[i] = w; w += L.b2; }
  a.Xg = reinterpret_cast<float*>(w); w += L.st;
  for (int i = 0; i < 2; ++i) { r.Sbuf[i] = reinterpret_cast<float*>(w); w += L.st; }
  a.Phi = reinterpret_cast<float*>(w); w += L.st;
  a.Plo = reinterpret_cast<float*>(w); w += L.st;
  a.Acc = reinterpret_cast<float*>(w); w += L.st;
  a.zhalf = L.zhalf;
  if (L.zhalf) { a.Zg = reinterpret_cast<float*>(w); w += L.st; }
  a.sb = ldexpf(1.f, d->scale_b_log2);
  a.inv_sb = ldexpf(1.f, -d->scale_b_log2);
  a.sy = ldexpf(1.f, d->scale_y_log2);
  a.inv_sy = ldexpf(1.f, -d->scale_y_log2);
  a.rk = sg::RK4{0, (float)(d->dt / 2.0), (float)d->dt, (float)(d->dt / 6.0),
                 (float)(d->dt / 6.0 - (double)(float)(d->dt / 6.0))};
  a.m = reinterpret_cast<const double2*>(d->m);
  a.m_stride = d->m_stride;
  a.mdg = d->m_diag;
  a.mdg_stride = d->m_diag_stride;
  if (a.mdg != nullptr) a.m = nullptr;
  a.keep_s = a.m != nullptr || a.mdg != nullptr;
  a.stage_store = nullptr;
  a.sb_exp_dev = nullptr;
  a.status = d->status;
  a.max_wait = 1u << 26;
  a.a1_bytes = L.a1; a.a2_bytes = L.a2; a.b1_bytes = L.b1; a.b2_bytes = L.b2;
  a.st_floats = L.st / sizeof(float);
  r.heff_t = reinterpret_cast<double2*>(reinterpret_cast<uint8_t*>(d->workspace) + L.total);

  const int per_g = L.MT1 * 128 + (K > 0 ? L.MT2 * 128 : 0);
  lsm::convert_kernel<<<G * per_g, 256, 0, st>>>(reinterpret_cast<const double2*>(d->heff), d->heff_stride,
                                                  reinterpret_cast<const double2*>(d->l_ops), d->l_stride, a, co, 0);
  LIME_CUDA_TRY(cudaGetLastError());
  ++launches;
  a.B1n[0] = r.B1[0][0]; a.B1n[1] = r.B1[0][1];
  a.Sn = r.Sbuf[0];
  const size_t runs = (size_t)r.B * L.W * (L.np / 8);
  const int eb = (int)((runs + 255) / 256 < 65535 ? (runs + 255) / 256 : 65535);
  lsm::init_kernel<<<eb, 256, 0, st>>>(a, reinterpret_cast<const double2*>(d->rho), r.B);
  LIME_CUDA_TRY(cudaGetLastError());
  ++launches;
  return LIME_OK;
}

int lsm_zlower_grid(const lsm::Args& a, int B) {
  const int xbs = a.np / 128;
  const size_t runs = (size_t)B * 2 * (xbs * (xbs - 1) / 2) * 128 * 16;
  const size_t g = (runs + 255) / 256;
  return (int)(g < 65535 ? (g > 0 ? g : 1) : 65535);
}

// stage s with stage-input buffers cur (read) and cur ^ 1 (written)
void lsm_bind_stage(LsmRun& r, int s, int cur) {
  r.a.rk.stage = s;
  r.a.B1c[0] = r.B1[cur][0]; r.a.B1c[1] = r.B1[cur][1];
  r.a.B1n[0] = r.B1[cur ^ 1][0]; r.a.B1n[1] = r.B1[cur ^ 1][1];
  r.a.Sc = r.Sbuf[cur];
  r.a.Sn = r.Sbuf[cur ^ 1];
}

int lsm_observe(const LimeLindbladStreamDesc* d, LsmRun& r, int step, cudaStream_t st, int64_t& launches) {
  const int obs_every = d->obs_every > 0 ? d->obs_every : 1;
  if (d->n_obs > 0 && ((step + 1) % obs_every) == 0) {
    lsm::observe_kernel<<<r.B * d->n_obs, 128, 0, st>>>(r.a, reinterpret_cast<const double2*>(d->obs_ops),
                                                        d->obs_stride, d->n_obs,
                                                        reinterpret_cast<double2*>(d->obs_out),
                                                        d->n_steps / obs_every, (step + 1) / obs_every - 1,
                                                        d->obs_diag);
    LIME_CUDA_TRY(cudaGetLastError());
    ++launches;
  }
  return LIME_OK;
}

int lsm_final(const LimeLindbladStreamDesc* d, LsmRun& r, cudaStream_t st, int64_t& launches) {
  const size_t tot = (size_t)r.B * d->n * d->n;
  const int fb = (int)((tot + 255) / 256 < 65535 ? (tot + 255) / 256 : 65535);
  lsm::final_kernel<<<fb, 256, 0, st>>>(r.a, reinterpret_cast<double2*>(d->rho), r.B);
  LIME_CUDA_TRY(cudaGetLastError());
  ++launches;
  return LIME_OK;
}

}  // namespace

extern "C" int lime_lindblad_rk4_stream(const LimeLindbladStreamDesc* d, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  int64_t launches = 0;
  LsmRun r;
  const int rc = lsm_prepare(d, r, st, launches);
  if (rc != LIME_OK) return rc;
  const LsmLayout& L = r.L;
  const int B = r.B, K = r.K, G = r.G;
  lsm::Args& a = r.a;
  const int tb = B * (L.np / 32) * (L.np / 32);            // 32 x 32 state tiles
  const size_t smem = sg::kSmemBytes;
  LIME_CUDA_TRY(cudaFuncSetAttribute(lsm::gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  LIME_CUDA_TRY(cudaFuncSetAttribute(lsm::gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int cur = 0;
  for (int step = 0; step < d->n_steps; ++step) {
    if (d->n_drive > 0) {
      // Heff(t) of this step, re-split into the GEMM 1 pieces
      const size_t tot = (size_t)G * d->n * d->n;
      const int hb = (int)((tot + 255) / 256 < 65535 ? (tot + 255) / 256 : 65535);
      lsm::heff_t_kernel<<<hb, 256, 0, st>>>(reinterpret_cast<const double2*>(d->heff), d->heff_stride, G, d->n,
                                             reinterpret_cast<const double2*>(d->drive_ops),
                                             d->drive_coef + (size_t)step * d->n_drive, d->n_drive, r.heff_t);
      LIME_CUDA_TRY(cudaGetLastError());
      lsm::convert_kernel<<<G * L.np, 256, 0, st>>>(r.heff_t, G == 1 ? 0 : (int64_t)d->n * d->n, nullptr, 0, a,
                                                    r.co, 1);
      LIME_CUDA_TRY(cudaGetLastError());
      launches += 2;
    }
    for (int s = 0; s < 4; ++s) {
      lsm_bind_stage(r, s, cur);
      lsm::gemm_kernel<false><<<B * L.MT1 * L.NT, sg::kThreads, smem, st>>>(a);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
      if (K > 0) {
        lsm::gemm_kernel<true><<<B * lsm::gemm2_tiles(a), sg::kThreads, smem, st>>>(a);
        if (a.zhalf) {
          LIME_CUDA_TRY(cudaGetLastError());
          lsm::zlower_kernel<<<lsm_zlower_grid(a, B), 256, 0, st>>>(a, B);
          ++launches;
        }
      } else {
        lsm::finish_kernel<<<tb, 256, 0, st>>>(a);
      }
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
      cur ^= 1;
    }
    const int orc = lsm_observe(d, r, step, st, launches);
    if (orc != LIME_OK) return orc;
  }
  const int frc = lsm_final(d, r, st, launches);
  if (frc != LIME_OK) return frc;
  count_launch(launches);
  return LIME_OK;
}

extern "C" int32_t lime_lindblad_stream_max_groups(void) { return lsm::kMaxGroups; }

extern "C" int lime_lindblad_rk4_stream_groups(const LimeLindbladStreamDesc* descs, int32_t n_groups,
                                               int32_t n_ctas, int32_t order, void* stream) {
  if (!descs || n_groups <= 0 || n_ctas < 0 || order < 0 || order > 1) return LIME_ERR_ARG;
  if (n_groups > lsm::kMaxGroups) return LIME_ERR_UNSUPPORTED;
  for (int i = 0; i < n_groups; ++i) {
    const LimeLindbladStreamDesc& d = descs[i];
    if (d.n_drive != 0) return LIME_ERR_UNSUPPORTED;
    if (d.n_steps != descs[0].n_steps || d.dt != descs[0].dt ||
        (d.obs_every > 0 ? d.obs_every : 1) != (descs[0].obs_every > 0 ? descs[0].obs_every : 1))
      return LIME_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int64_t launches = 0;
  LsmRun runs[lsm::kMaxGroups];
  for (int i = 0; i < n_groups; ++i) {
    const int rc = lsm_prepare(&descs[i], runs[i], st, launches);
    if (rc != LIME_OK) return rc;
  }
  int dev = 0, sms = 0;
  LIME_CUDA_TRY(cudaGetDevice(&dev));
  LIME_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t smem = sg::kSmemBytes;
  LIME_CUDA_TRY(cudaFuncSetAttribute(lsm::gemm_groups_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
  LIME_CUDA_TRY(cudaFuncSetAttribute(lsm::gemm_groups_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
  // tile lists: groups by decreasing chunks per tile (order 1), or as given (order 0)
  int ord1[lsm::kMaxGroups], ord2[lsm::kMaxGroups];
  int n2 = 0;
  for (int i = 0; i < n_groups; ++i) {
    ord1[i] = i;
    if (runs[i].K > 0) ord2[n2++] = i;
  }
  if (order == 1) {
    auto sort_by = [&](int* o, int cnt, bool z) {
      for (int i = 1; i < cnt; ++i)
        for (int j = i; j > 0; --j) {
          const int kj = z ? runs[o[j]].L.KC2 : runs[o[j]].L.KC1;
          const int kp = z ? runs[o[j - 1]].L.KC2 : runs[o[j - 1]].L.KC1;
          if (kj > kp) { const int tmp = o[j]; o[j] = o[j - 1]; o[j - 1] = tmp; } else break;
        }
    };
    sort_by(ord1, n_groups, false);
    sort_by(ord2, n2, true);
  }
  auto fill = [&](lsm::Groups& m, const int* o, int cnt, bool z) {
    m.n_groups = cnt;
    m.start[0] = 0;
    for (int i = 0; i < cnt; ++i) {
      const LsmRun& r = runs[o[i]];
      m.g[i] = r.a;
      m.start[i + 1] = m.start[i] + r.B * (z ? lsm::gemm2_tiles(r.a) : r.L.MT1 * r.L.NT);
    }
    m.n_items = m.start[cnt];
  };
  auto grid_of = [&](int items) {
    const int g = n_ctas > 0 ? n_ctas : sms;
    return g < items ? g : items;
  };
  lsm::Groups m1, m2;   // launch parameters (copied at each launch)
  int cur = 0;
  for (int step = 0; step < descs[0].n_steps; ++step) {
    for (int s = 0; s < 4; ++s) {
      for (int i = 0; i < n_groups; ++i) lsm_bind_stage(runs[i], s, cur);
      fill(m1, ord1, n_groups, false);
      lsm::gemm_groups_kernel<false><<<grid_of(m1.n_items), sg::kThreads, smem, st>>>(m1);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
      if (n2 > 0) {
        fill(m2, ord2, n2, true);
        lsm::gemm_groups_kernel<true><<<grid_of(m2.n_items), sg::kThreads, smem, st>>>(m2);
        LIME_CUDA_TRY(cudaGetLastError());
        ++launches;
        for (int i = 0; i < n_groups; ++i) {
          if (runs[i].K == 0 || !runs[i].a.zhalf) continue;
          lsm::zlower_kernel<<<lsm_zlower_grid(runs[i].a, runs[i].B), 256, 0, st>>>(runs[i].a, runs[i].B);
          LIME_CUDA_TRY(cudaGetLastError());
          ++launches;
        }
      }
      for (int i = 0; i < n_groups; ++i) {
        if (runs[i].K > 0) continue;
        const int tb = runs[i].B * (runs[i].L.np / 32) * (runs[i].L.np / 32);
        lsm::finish_kernel<<<tb, 256, 0, st>>>(runs[i].a);
        LIME_CUDA_TRY(cudaGetLastError());
        ++launches;
      }
      cur ^= 1;
    }
    for (int i = 0; i < n_groups; ++i) {
      const int orc = lsm_observe(&descs[i], runs[i], step, st, launches);
      if (orc != LIME_OK) return orc;
    }
  }
  for (int i = 0; i < n_groups; ++i) {
    const int frc = lsm_final(&descs[i], runs[i], st, launches);
    if (frc != LIME_OK) return frc;
  }
  count_launch(launches);
  return LIME_OK;
}

extern "C" size_t lime_lindblad_adjoint_stream_workspace(int32_t n, int32_t batch, int32_t n_generators,
                                                         int32_t seg_steps) {
  if (n <= 0 || batch <= 0 || n_generators <= 0 || seg_steps <= 0) return 0;
  const LsmLayout L = lsm_layout(n, batch, n_generators, 0);
  return L.total + 3 * L.a1 + L.r1 + 3 * L.st + 1024 + 4 * (size_t)seg_steps * L.st;
}

extern "C" int lime_lindblad_adjoint_stream(const LimeLindbladAdjointStreamDesc* d, void* stream) {
  if (!d || d->n <= 0 || d->batch <= 0 || d->n_steps <= 0 || d->seg_steps <= 0 || d->n_obs < 0) return LIME_ERR_ARG;
  if (!d->ckpt || !d->heff || !d->heff_adj || !d->grad_diag || !d->grad_bond || !d->grad_gamma) return LIME_ERR_ARG;
  if (!d->workspace || !d->status) return LIME_ERR_ARG;
  if (d->n_obs > 0 && (!d->obs_ops || !d->obs_grad)) return LIME_ERR_ARG;
  if ((d->m == nullptr) != (d->m_adj == nullptr)) return LIME_ERR_ARG;
  if (d->heff_stride < 0 || d->heff_adj_stride < 0 || d->m_stride < 0 || d->obs_stride < 0) return LIME_ERR_ARG;
  if (d->m_diag_stride < 0) return LIME_ERR_ARG;
  if (d->scale_b_log2 < -60 || d->scale_b_log2 > 60 || d->scale_l_log2 < -60 || d->scale_l_log2 > 60)
    return LIME_ERR_ARG;
  if (d->n > 4096) return LIME_ERR_UNSUPPORTED;
  const int P = d->param_batch > 0 ? d->param_batch : d->batch;
  if (P > d->batch) return LIME_ERR_ARG;
  const int obs_every = d->obs_every > 0 ? d->obs_every : 1;
  const int G = (d->heff_stride == 0 && d->heff_adj_stride == 0) ? 1 : P;
  const int seg = d->seg_steps;
  if (d->workspace_bytes < lime_lindblad_adjoint_stream_workspace(d->n, d->batch, G, seg)) return LIME_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(d->workspace) & 1023) != 0) return LIME_ERR_ARG;
  const LsmLayout L = lsm_layout(d->n, d->batch, G, 0);
  const int B = d->batch;
  cudaStream_t st = (cudaStream_t)stream;

  uint8_t* w = reinterpret_cast<uint8_t*>(d->workspace);
  lsm::Args af{};
  lsm::ConvertOut cf{}, ca{};
  af.n = d->n; af.np = L.np; af.W = L.W; af.NT = L.NT; af.K = 0; af.P = P; af.G = G;
  af.KC1 = L.KC1; af.KC2 = 0; af.MT1 = L.MT1; af.MT2 = 0;
  for (int i = 0; i < 3; ++i) { af.A1[i] = cf.A1[i] = w; w += L.a1; }
  for (int i = 0; i < 3; ++i) { af.A2[i] = cf.A2[i] = w; w += L.a2; }
  af.rinv1 = cf.rinv1 = reinterpret_cast<float*>(w); w += L.r1;
  af.rinv2 = cf.rinv2 = reinterpret_cast<float*>(w); w += L.r2;
  uint8_t* B1[2][2];
  for (int bb = 0; bb < 2; ++bb)
    for (int i = 0; i < 2; ++i) { B1[bb][i] = w; w += L.b1; }
  for (int i = 0; i < 2; ++i) { af.B2[i] = w; w += L.b2; }
  af.Xg = reinterpret_cast<float*>(w); w += L.st;
  float* Sbuf[2];
  for (int i = 0; i < 2; ++i) { Sbuf[i] = reinterpret_cast<float*>(w); w += L.st; }
  af.Phi = reinterpret_cast<float*>(w); w += L.st;
  af.Plo = reinterpret_cast<float*>(w); w += L.st;
  af.Acc = reinterpret_cast<float*>(w); w += L.st;
  w = reinterpret_cast<uint8_t*>(d->workspace) + L.total;   // past the forward layout (and its slack)
  af.a1_bytes = L.a1; af.a2_bytes = L.a2; af.b1_bytes = L.b1; af.b2_bytes = L.b2;
  af.st_floats = L.st / sizeof(float);
  lsm::Args aa = af;                                          // the adjoint generator: own A pieces
  for (int i = 0; i < 3; ++i) { aa.A1[i] = ca.A1[i] = w; w += L.a1; }
  aa.rinv1 = ca.rinv1 = reinterpret_cast<float*>(w); w += L.r1;
  lsm::AdjState J{};
  J.Lhi = reinterpret_cast<float*>(w); w += L.st;
  J.Llo = reinterpret_cast<float*>(w); w += L.st;
  J.LAcc = reinterpret_cast<float*>(w); w += L.st;
  J.lmax = reinterpret_cast<unsigned*>(w);
  J.sl_exp = reinterpret_cast<int*>(w + 4);
  w += 1024;
  float* store = reinterpret_cast<float*>(w);                 // [seg][4][B][W][np]
  const size_t inst = (size_t)L.W * L.np;

  af.sb = ldexpf(1.f, d->scale_b_log2);
  af.inv_sb = ldexpf(1.f, -d->scale_b_log2);
  aa.sb = aa.inv_sb = 1.f;                                    // (per step: J.sl_exp)
  J.bound = (float)(d->dt / 2.0);
  af.rk = sg::RK4{0, (float)(d->dt / 2.0), (float)d->dt, (float)(d->dt / 6.0),
                  (float)(d->dt / 6.0 - (double)(float)(d->dt / 6.0))};
  af.m = reinterpret_cast<const double2*>(d->m);
  aa.m = reinterpret_cast<const double2*>(d->m_adj);
  af.m_stride = aa.m_stride = d->m_stride;
  // a real diagonal M is its own conjugate: both directions use it
  af.mdg = aa.mdg = d->m_diag;
  af.mdg_stride = aa.mdg_stride = d->m_diag_stride;
  if (d->m_diag != nullptr) af.m = aa.m = nullptr;
  af.keep_s = aa.keep_s = true;
  af.sb_exp_dev = nullptr;
  aa.sb_exp_dev = J.sl_exp;
  af.stage_store = aa.stage_store = nullptr;
  af.status = aa.status = d->status;
  af.max_wait = aa.max_wait = 1u << 26;
  int64_t launches = 0;

  const int per_g = L.MT1 * 128;
  lsm::convert_kernel<<<G * per_g, 256, 0, st>>>(reinterpret_cast<const double2*>(d->heff), d->heff_stride,
                                                  nullptr, 0, af, cf, 0);
  LIME_CUDA_TRY(cudaGetLastError());
  lsm::convert_kernel<<<G * per_g, 256, 0, st>>>(reinterpret_cast<const double2*>(d->heff_adj),
                                                  d->heff_adj_stride, nullptr, 0, aa, ca, 0);
  LIME_CUDA_TRY(cudaGetLastError());
  launches += 2;
  LIME_CUDA_TRY(cudaMemsetAsync(J.Lhi, 0, 2 * L.st, st));   // Lhi and Llo
  LIME_CUDA_TRY(cudaMemsetAsync(J.lmax, 0, 8, st));          // lmax and sl_exp
  const size_t smem = sg::kSmemBytes;
  LIME_CUDA_TRY(cudaFuncSetAttribute(lsm::gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const size_t runs = (size_t)B * L.W * (L.np / 8);
  const int eb = (int)((runs + 255) / 256 < 65535 ? (runs + 255) / 256 : 65535);
  const int tb = B * (L.np / 32) * (L.np / 32);            // 32 x 32 state tiles
  const int gemm_grid = B * L.MT1 * L.NT;
  const int n_slots = d->n_steps / obs_every;
  const int n_seg = (d->n_steps + seg - 1) / seg;
  const double dt = d->dt;

  for (int sgi = n_seg - 1; sgi >= 0; --sgi) {
    const int s0 = sgi * seg;
    const int len = (d->n_steps - s0 < seg) ? d->n_steps - s0 : seg;
    // ---- forward recompute of the segment, storing every stage input
    int cur = 0;
    af.B1n[0] = B1[0][0]; af.B1n[1] = B1[0][1];
    af.Sn = Sbuf[0];
    lsm::init_kernel<<<eb, 256, 0, st>>>(af, reinterpret_cast<const double2*>(d->ckpt) + (size_t)sgi * B * d->n * d->n,
                                         B);
    LIME_CUDA_TRY(cudaGetLastError());
    ++launches;
    for (int s = 0; s < len; ++s) {
      for (int k = 0; k < 4; ++k) {
        af.rk.stage = k;
        af.B1c[0] = B1[cur][0]; af.B1c[1] = B1[cur][1];
        af.B1n[0] = B1[cur ^ 1][0]; af.B1n[1] = B1[cur ^ 1][1];
        af.Sc = Sbuf[cur];
        af.Sn = Sbuf[cur ^ 1];
        af.stage_store = store + ((size_t)s * 4 + k) * B * inst;
        lsm::gemm_kernel<false><<<gemm_grid, sg::kThreads, smem, st>>>(af);
        LIME_CUDA_TRY(cudaGetLastError());
        lsm::finish_kernel<<<tb, 256, 0, st>>>(af);
        LIME_CUDA_TRY(cudaGetLastError());
        launches += 2;
        cur ^= 1;
      }
    }
    af.stage_store = nullptr;
    // ---- backward through the segment
    int c = 0;
    for (int s = len - 1; s >= 0; --s) {
      const int gstep = s0 + s;
      const int slot = (d->n_obs > 0 && ((gstep + 1) % obs_every) == 0) ? (gstep + 1) / obs_every - 1 : -1;
      aa.B1n[0] = B1[c][0]; aa.B1n[1] = B1[c][1];
      aa.Sn = Sbuf[c];
      lsm::adj_source_kernel<<<eb, 256, 0, st>>>(aa, J, B, reinterpret_cast<const double2*>(d->obs_ops),
                                                  d->obs_stride, d->n_obs,
                                                  reinterpret_cast<const double2*>(d->obs_grad), n_slots, slot,
                                                  reinterpret_cast<const float2*>(d->obs_coef));
      LIME_CUDA_TRY(cudaGetLastError());
      lsm::adj_scale_kernel<<<1, 1, 0, st>>>(J);
      LIME_CUDA_TRY(cudaGetLastError());
      lsm::adj_start_kernel<<<eb, 256, 0, st>>>(aa, J, B, (float)(dt / 6.0));
      LIME_CUDA_TRY(cudaGetLastError());
      launches += 3;
      for (int i = 4; i >= 1; --i) {
        aa.B1c[0] = B1[c][0]; aa.B1c[1] = B1[c][1];
        aa.Sc = Sbuf[c];
        aa.B1n[0] = B1[c ^ 1][0]; aa.B1n[1] = B1[c ^ 1][1];
        aa.Sn = Sbuf[c ^ 1];
        lsm::gemm_kernel<false><<<gemm_grid, sg::kThreads, smem, st>>>(aa);
        LIME_CUDA_TRY(cudaGetLastError());
        lsm::adj_grad_kernel<<<B * (L.np / 8), 128, 0, st>>>(aa, Sbuf[c], store + ((size_t)s * 4 + (i - 1)) * B * inst,
                                                             B, d->grad_diag, d->grad_bond, d->grad_gamma);
        LIME_CUDA_TRY(cudaGetLastError());
        const float c_l = (float)(i == 2 ? dt / 6.0 : dt / 3.0);
        const float c_y = (float)(i == 4 ? dt : dt / 2.0);
        lsm::adj_finish_kernel<<<tb, 256, 0, st>>>(aa, J, i, c_l, c_y);
        LIME_CUDA_TRY(cudaGetLastError());
        launches += 3;
        if (i > 1) c ^= 1;
      }
    }
  }
  if (d->lam) {
    lsm::Args al = af;
    al.Phi = J.Lhi;
    al.Plo = J.Llo;
    const size_t tot = (size_t)B * d->n * d->n;
    const int fb = (int)((tot + 255) / 256 < 65535 ? (tot + 255) / 256 : 65535);
    lsm::final_kernel<<<fb, 256, 0, st>>>(al, reinterpret_cast<double2*>(d->lam), B);
    LIME_CUDA_TRY(cudaGetLastError());
    ++launches;
  }
  count_launch(launches);
  return LIME_OK;
}
