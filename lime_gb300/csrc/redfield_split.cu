// Split-precision Bloch-Redfield RK4 on the sm_103a tensor cores (tcgen05).
//
// Per RK4 stage the generator application over the right-hand-side block is
// one large complex GEMM Y = L S (L: D x D, S: D x R).  It runs as the real
// GEMM
//     [Yr | Yi] (D x 2R) = [Lr | Li] (D x 2D) . [[Sr, Si], [-Si, Sr]] (2D x 2R)
// so the big operand L is streamed once per stage without duplication, on
// the streaming split-precision tile of stream_gemm.cuh (bulk-copy operand
// ring, exact dominant product, fp32 two-sum accumulation).
//
// RK4 state (lime/oqs.py:453-462, lime/phys.py:636-649): P = hi + lo fp32
// and the stage accumulator, component-planar [2R][D] (column jj < R is
// Re vec rho_jj, jj >= R is Im vec rho_{jj-R}); the tile's epilogue updates
// the state in 8-row runs and writes the next stage input straight into the
// other B buffer as 16-byte stores (ping-pong across stages).  Observables
// are a second GEMM of the same form with A = the observables, K split over
// CTAs whose partial sums are added atomically in fp64.

#include "stream_gemm.cuh"

namespace lime {
namespace rsp {

using sg::kBM;
using sg::kBN;
using sg::kFStride;
using sg::kGroup;
using sg::kPiece;

struct StageArgs {
  int Dp, W, KC, MT, NT, stage;      // W = 2 Rp output columns, KC = 2Dp / kCK chunks, NT = W / 128
  int KS, groups_per_split;          // observable pass: K split over KS CTAs, 128-K groups each
  float inv_sb, sb, c_half, c_full, c_sixth, c_sixth_lo;
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
  // extents for the bounds-checked build: bytes of one A and one B piece
  // buffer, floats of one state array
  size_t a_bytes = kNoExtent, b_bytes = kNoExtent, st_floats = kNoExtent;
};

// kObserve = false: one RK4 stage, Y = L S over the full K, fused stage
// update.  kObserve = true: observables <E_o> = sum_d Et[o][d] P[d][r] of
// the state held in Bc, K split over KS CTAs.
template <bool kObserve>
__global__ void __launch_bounds__(sg::kThreads, 1) gemm_kernel(StageArgs a) {
  extern __shared__ uint8_t smem_raw[];
  sg::Smem& S = *reinterpret_cast<sg::Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int t = threadIdx.x, lane = t & 31;
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
  sg::setup(S);
  sg::Tile T;
  for (int i = 0; i < 3; ++i) T.A[i] = a.A[i] + (size_t)mt * a.KC * kPiece;
  for (int i = 0; i < 2; ++i) T.B[i] = a.Bc[i] + (size_t)nt * a.KC * kPiece;
  T.c0 = c0;
  T.n_chunks = KC;
  T.row_inv = a.row_inv + (size_t)mt * kBM;
  T.inv_sb = a.inv_sb;
  T.max_wait = a.max_wait;
  T.a_avail = a.a_bytes - (size_t)mt * a.KC * kPiece;
  T.b_avail = a.b_bytes - (size_t)nt * a.KC * kPiece;
  T.status = a.status;
  const float* ft = S.tile();
  if (sg::mainloop(S, T) && !*(volatile int*)&S.abort) {
    const int u = t - sg::kEpiFirst, ew = u >> 5;
    if (kObserve) {
      // row r = observable, kEpiCols columns per thread
      const int r = u & 127, hh = u >> 7;
      const int o = mt * kBM + r;
      if (o < a.n_obs && KC > 0) {
#pragma unroll 4
        for (int c = 0; c < sg::kEpiCols; ++c) {
          const int jj = nt * kBN + sg::kEpiCols * hh + c;
          const int j = jj < a.Rp ? jj : jj - a.Rp;
          if (j < a.R)
            atomicAdd(a.obs + 2 * ((size_t)j * a.n_obs + o) + (jj < a.Rp ? 0 : 1),
                      (double)ft[(sg::kEpiCols * hh + c) * kFStride + r]);
        }
      }
    } else {
      // ---- fused RK4 stage update in runs of 8 rows: lane -> (column & 7, row run & 3)
      const int nlo = lane & 7, glo = lane >> 3;
      const sg::RK4 k4{a.stage, a.c_half, a.c_full, a.c_sixth, a.c_sixth_lo};
      bool bad = false, range = false;
#pragma unroll 1
      for (int wi = ew; wi < 64; wi += sg::kEpiWarps) {
        const int jl = (wi >> 2) * 8 + nlo;
        const int dl = ((wi & 3) * 4 + glo) * 8;
        const int jj = nt * kBN + jl, d = mt * kBM + dl;
        float f[8], sv[8];
        if (!in_bounds(((size_t)jj * a.Dp + d) * sizeof(float), 8 * sizeof(float), a.st_floats * sizeof(float),
                       a.status))
          continue;
        sg::ld8(ft + jl * kFStride + dl, f);
        sg::rk4_stage8(k4, a.Phi, a.Plo, a.Acc, (size_t)jj * a.Dp + d, f, sv, bad);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          sv[i] = __fmul_rn(sv[i], a.sb);
          range |= !(fabsf(sv[i]) <= sg::kBMax);
        }
        const bool im = jj >= a.Rp;
        sg::scatter_cplx8(a.Bn[0], a.Bn[1], a.KC, a.Dp, a.Rp, d, im ? jj - a.Rp : jj, im, sv, a.b_bytes, a.status);
      }
      if (bad) atomicOr(a.status, LIME_FLAG_NONFINITE);
      if (range) atomicOr(a.status, LIME_FLAG_RANGE);
    }
  }
  sg::teardown(S, a.status);
}

// A pieces of generator rows (transposed = 0: element (row, kk) = L[row][kk])
// or of observables (transposed = 1: element (o, a n + b) = E_o[b][a], so
// that <E_o> = sum_d M[o][d] vec(rho)[d]).
__global__ void convert_rows_kernel(const double2* M, int transposed, int n, int rows, int D, int Dp, int KC,
                                    uint8_t* A0, uint8_t* A1, uint8_t* A2, float* row_inv) {
  const int row = blockIdx.x;
  auto elem = [&](int kk) -> double2 {
    if (!transposed) return M[(size_t)row * D + kk];
    const int ia = kk / n, ib = kk - ia * n;
    return M[(size_t)row * D + (size_t)ib * n + ia];
  };
  sg::convert_row(elem, row, row < rows, D, Dp, KC, A0, A1, A2, row_inv);
}

// state from complex128 rho [R][D] (row-major vec per RHS) and the first B
// input; one thread per run of 8 rows of one column
__global__ void init_state_kernel(StageArgs a, const double2* rho, int D, int R) {
  const size_t total = (size_t)a.W * (a.Dp / 8);
  bool range = false;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
    const int jj = (int)(g / (a.Dp / 8)), d = (int)(g % (a.Dp / 8)) * 8;
    const bool im = jj >= a.Rp;
    const int j = im ? jj - a.Rp : jj;
    float hv[8], lv[8], x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      double v = 0.0;
      if (d + i < D && j < R) {
        const double2 z = rho[(size_t)j * D + d + i];
        v = im ? z.y : z.x;
      }
      hv[i] = (float)v;
      lv[i] = (float)(v - (double)hv[i]);
      x[i] = __fmul_rn(hv[i], a.sb);
      range |= !(fabsf(x[i]) <= sg::kBMax);
    }
    const size_t e = (size_t)jj * a.Dp + d;
    sg::st8(a.Phi + e, hv);
    sg::st8(a.Plo + e, lv);
    sg::scatter_cplx8(a.Bn[0], a.Bn[1], a.KC, a.Dp, a.Rp, d, j, im, x, a.b_bytes, a.status);
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
  KC = 2 * Dp / sg::kCK;
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
  l.apiece = (size_t)MT * KC * sg::kPiece;
  l.epiece = (size_t)MTo * KC * sg::kPiece;
  l.bpiece = (size_t)NT * KC * sg::kPiece;
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
  a.KS = 1; a.groups_per_split = KC / sg::kGroup;
  a.inv_sb = ldexpf(1.f, -d->scale_b_log2);
  a.sb = ldexpf(1.f, d->scale_b_log2);
  a.c_half = (float)(d->dt / 2.0);
  a.c_full = (float)d->dt;
  a.c_sixth = (float)(d->dt / 6.0);
  a.c_sixth_lo = (float)(d->dt / 6.0 - (double)a.c_sixth);
  a.A[0] = A[0]; a.A[1] = A[1]; a.A[2] = A[2];
  a.row_inv = row_inv;
  a.Phi = Phi; a.Plo = Plo; a.Acc = Acc;
  a.status = d->status;
  a.max_wait = 1u << 26;
  a.a_bytes = L.apiece; a.b_bytes = L.bpiece; a.st_floats = (size_t)W * Dp;
  // first B input = rho0
  a.Bn[0] = B[0]; a.Bn[1] = B[1];
  const size_t tot = (size_t)W * Dp;
  const int ib = (int)((tot / 8 + 255) / 256);
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
    ao.a_bytes = L.epiece;
    ao.row_inv = row_inv + (size_t)MT * 128;
    ao.n_obs = d->n_obs;
    const int groups = KC / sg::kGroup;
    int ks = (2 * n_sm) / (MTo * NT);
    ks = ks < 1 ? 1 : (ks > groups ? groups : ks);
    ao.groups_per_split = (groups + ks - 1) / ks;
    ao.KS = (groups + ao.groups_per_split - 1) / ao.groups_per_split;
  }

  const size_t smem = sg::kSmemBytes;
  LIME_CUDA_TRY(cudaFuncSetAttribute(rsp::gemm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  LIME_CUDA_TRY(cudaFuncSetAttribute(rsp::gemm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int obs_every = d->obs_every > 0 ? d->obs_every : 1;
  int cur = 0;   // B[2cur], B[2cur+1] hold the current stage input
  for (int step = 0; step < d->n_steps; ++step) {
    for (int s = 0; s < 4; ++s) {
      a.stage = s;
      a.Bc[0] = B[2 * cur]; a.Bc[1] = B[2 * cur + 1];
      a.Bn[0] = B[2 * (cur ^ 1)]; a.Bn[1] = B[2 * (cur ^ 1) + 1];
      rsp::gemm_kernel<false><<<MT * NT, sg::kThreads, smem, st>>>(a);
      LIME_CUDA_TRY(cudaGetLastError());
      ++launches;
      cur ^= 1;
    }
    if (MTo > 0 && ((step + 1) % obs_every) == 0) {
      // B[2cur], B[2cur+1] now hold the new state (the next step's stage-0 input)
      const int slot = (step + 1) / obs_every - 1;
      ao.Bc[0] = B[2 * cur]; ao.Bc[1] = B[2 * cur + 1];
      ao.obs = d->obs_out + (size_t)slot * d->n_rhs * d->n_obs * 2;
      rsp::gemm_kernel<true><<<ao.KS * MTo * NT, sg::kThreads, smem, st>>>(ao);
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
