// Self-tests of the bounded device-side waits (test infrastructure; no
// propagation).  Every wait in the propagator kernels polls an mbarrier at
// most max_wait times; when the phase never completes the kernel ORs
// LIME_FLAG_TIMEOUT into its status word, releases what it holds and
// returns, so the context stays usable.  These kernels make such waits run
// out on purpose — on a barrier that nothing completes, or in the streaming
// GEMM tile with its operand copies withheld — next to controls in which
// the waits complete.  Kind 4 (bounds-checked build only) refuses an
// operand copy whose declared extent is too short and reports
// LIME_FLAG_BOUNDS.

#include "stream_gemm.cuh"

namespace lime {
namespace selftest {

constexpr int kTileChunks = 2;
constexpr size_t kTileBytes = (size_t)5 * kTileChunks * sg::kPiece + 128 * sizeof(float);

__global__ void mbar_kernel(int arrive, uint32_t max_wait, int32_t* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  __syncthreads();
  if (arrive && threadIdx.x == 0) tc::mbar_arrive(&bar);
  if (!tc::mbar_wait_bounded(&bar, 0u, max_wait)) atomicOr(status, LIME_FLAG_TIMEOUT);
}

// One 128 x 128 tile of zero operands over two K chunks; the parked result
// must be zero.
// short_extent (bounds-checked build): the tile is told its A operand holds
// one piece fewer than the two chunks it reads, so the producer's extent
// check refuses the second copy (no access leaves the buffer) and the tile
// aborts.
__global__ void __launch_bounds__(sg::kThreads, 1)
    tile_kernel(const uint8_t* ws, int withhold, int short_extent, uint32_t max_wait, int32_t* status) {
  extern __shared__ uint8_t smem_raw[];
  sg::Smem& S = *reinterpret_cast<sg::Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  sg::setup(S);
  sg::Tile T;
  for (int i = 0; i < 3; ++i) T.A[i] = ws + (size_t)i * kTileChunks * sg::kPiece;
  for (int i = 0; i < 2; ++i) T.B[i] = ws + (size_t)(3 + i) * kTileChunks * sg::kPiece;
  T.c0 = 0;
  T.n_chunks = kTileChunks;
  T.row_inv = reinterpret_cast<const float*>(ws + (size_t)5 * kTileChunks * sg::kPiece);
  T.inv_sb = 1.f;
  T.max_wait = max_wait;
  T.withhold = withhold;
  T.a_avail = short_extent ? (size_t)(kTileChunks - 1) * sg::kPiece : (size_t)kTileChunks * sg::kPiece;
  T.b_avail = (size_t)kTileChunks * sg::kPiece;
  T.status = status;
  if (sg::mainloop(S, T) && !*(volatile int*)&S.abort) {
    const int u = threadIdx.x - sg::kEpiFirst;
    const float* ft = S.tile();
    bool nonzero = false;
    for (int e = u; e < sg::kBM * sg::kBN; e += sg::kEpiThreads)
      nonzero |= ft[(e / sg::kBM) * sg::kFStride + (e % sg::kBM)] != 0.f;
    if (nonzero) atomicOr(status, LIME_FLAG_NONFINITE);
  }
  sg::teardown(S, status);
}

}  // namespace selftest
}  // namespace lime

using namespace lime;

extern "C" size_t lime_wait_selftest_workspace(void) { return selftest::kTileBytes; }

extern "C" int lime_wait_selftest(int kind, uint32_t max_wait, const void* ws, int32_t* status, void* stream) {
  if (kind < 0 || kind > 4 || !status || max_wait == 0) return LIME_ERR_ARG;
#ifndef LIME_CHECK
  if (kind == 4) return LIME_ERR_UNSUPPORTED;   // the extent check exists only in the bounds-checked build
#endif
  if (kind >= 2 && (!ws || (reinterpret_cast<uintptr_t>(ws) & 15) != 0)) return LIME_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  if (kind < 2) {
    selftest::mbar_kernel<<<1, 64, 0, st>>>(kind == 1, max_wait, status);
  } else {
    LIME_CUDA_TRY(cudaFuncSetAttribute(selftest::tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)sg::kSmemBytes));
    selftest::tile_kernel<<<1, sg::kThreads, sg::kSmemBytes, st>>>(static_cast<const uint8_t*>(ws), kind == 2,
                                                                    kind == 4, max_wait, status);
  }
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch();
  return LIME_OK;
}
