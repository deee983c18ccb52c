// Batched complex128 discrete Fourier transforms for the spectra of
// propagated correlation functions (lime/fft.py:9-56: g(w) = fftshift(fft(f))
// dx exp(-i w x0)).  Power-of-two lengths up to 8192 run as one CTA per
// transform, radix-2 decimation in time entirely in shared memory (inputs
// loaded in bit-reversed order, log2 n butterfly stages, twiddles from
// sincospi); other lengths up to 4096 go through Bluestein's chirp-z
// identity
//     X_k = c_k sum_j (x_j c_j) conj(c_{k-j}),   c_j = exp(-i pi j^2 / n)
// as a circular convolution of length m = 2^ceil(log2(2n - 1)) (three
// power-of-two transforms).  The output can be written fftshift-ed and
// multiplied by a per-position factor (dx exp(-i w_k x0) for lime's fft).

#include "common.cuh"

namespace lime {
namespace fft {

constexpr int kThreads = 512;
constexpr int kMaxPow2 = 8192;

struct Pass {
  int n, log2n, inverse;
  const double2* x; int64_t x_s, x_bs;
  double2* y; int64_t y_s, y_bs;
  int shift;                 // write output k at (k + n/2) % n
  const double2* post;       // per output position factor (after the shift), or null
  const double2* mul;        // per frequency factor applied before the store (Bluestein's B_k), or null
  double scale;
};

__device__ __forceinline__ unsigned bitrev(unsigned v, int bits) { return bits == 0 ? 0u : __brev(v) >> (32 - bits); }

__global__ void __launch_bounds__(kThreads) pow2_kernel(Pass p) {
  extern __shared__ double2 s[];
  const int n = p.n;
  const int64_t b = blockIdx.x;
  const double2* x = p.x + b * p.x_bs;
  for (int j = threadIdx.x; j < n; j += kThreads) s[bitrev((unsigned)j, p.log2n)] = x[(int64_t)j * p.x_s];
  __syncthreads();
  const double sgn = p.inverse ? 1.0 : -1.0;
  for (int half = 1; half < n; half <<= 1) {
    for (int q = threadIdx.x; q < n / 2; q += kThreads) {
      const int pos = q & (half - 1);
      const int i0 = ((q - pos) << 1) + pos, i1 = i0 + half;
      double sn, cs;
      sincospi(sgn * (double)pos / (double)half, &sn, &cs);   // exp(-+ i pi pos / half)
      const double2 u = s[i0], v = s[i1];
      const double2 w = make_double2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
      s[i0] = make_double2(u.x + w.x, u.y + w.y);
      s[i1] = make_double2(u.x - w.x, u.y - w.y);
    }
    __syncthreads();
  }
  double2* y = p.y + b * p.y_bs;
  for (int k = threadIdx.x; k < n; k += kThreads) {
    double2 v = s[k];
    if (p.mul) v = cmul(v, p.mul[k]);
    v = cscale(v, p.scale);
    const int ks = p.shift ? (k + n / 2) % n : k;
    if (p.post) v = cmul(v, p.post[ks]);
    y[(int64_t)ks * p.y_s] = v;
  }
}

// exp(sgn i pi j^2 / n) with the argument reduced exactly (j^2 mod 2n)
__device__ __forceinline__ double2 chirp(int64_t j, int n, double sgn) {
  const int64_t r = (j * j) % (2 * (int64_t)n);
  double sn, cs;
  sincospi(sgn * (double)r / (double)n, &sn, &cs);
  return make_double2(cs, sn);
}

// a[b][j] = x[b][j] c_j (j < n), 0 up to m
__global__ void chirp_in_kernel(const double2* x, int64_t x_s, int64_t x_bs, int n, int m, int batch, double sgn,
                                double2* a) {
  const int64_t total = (int64_t)batch * m;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / m;
    const int j = (int)(e - b * m);
    a[e] = j < n ? cmul(x[b * x_bs + (int64_t)j * x_s], chirp(j, n, sgn)) : cz();
  }
}

// the chirp filter conj(c_m), wrapped circularly into length m
__global__ void chirp_filter_kernel(int n, int m, double sgn, double2* f) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    double2 v = cz();
    if (k < n) v = chirp(k, n, -sgn);
    else if (k > m - n) v = chirp(m - k, n, -sgn);
    f[k] = v;
  }
}

// X_k = c_k conv_k / m, written (shifted, times post) to y
__global__ void chirp_out_kernel(const double2* conv, int n, int m, int batch, double sgn, int shift,
                                 const double2* post, double2* y, int64_t y_s, int64_t y_bs) {
  const int64_t total = (int64_t)batch * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / n;
    const int k = (int)(e - b * n);
    double2 v = cscale(cmul(conv[b * m + k], chirp(k, n, sgn)), 1.0 / (double)m);
    const int ks = shift ? (k + n / 2) % n : k;
    if (post) v = cmul(v, post[ks]);
    y[b * y_bs + (int64_t)ks * y_s] = v;
  }
}

int log2_exact(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return (1 << l) == n ? l : -1;
}

int bluestein_len(int n) {
  int m = 1;
  while (m < 2 * n - 1) m <<= 1;
  return m;
}

}  // namespace fft
}  // namespace lime

using namespace lime;

extern "C" size_t lime_fft_f64_workspace(int32_t n, int32_t batch) {
  if (n <= 0 || batch <= 0) return 0;
  if (fft::log2_exact(n) >= 0) return 0;
  const int m = fft::bluestein_len(n);
  return ((size_t)batch + 1) * m * sizeof(double2);
}

extern "C" int lime_fft_f64(const LimeFftDesc* d, void* stream) {
  if (!d || d->n <= 0 || d->batch <= 0 || !d->x || !d->y) return LIME_ERR_ARG;
  if ((d->inverse & ~1) || (d->shift & ~1)) return LIME_ERR_ARG;
  const int n = d->n;
  cudaStream_t st = (cudaStream_t)stream;
  const double sgn = d->inverse ? 1.0 : -1.0;
  const size_t smem_max = (size_t)fft::kMaxPow2 * sizeof(double2);
  LIME_CUDA_TRY(cudaFuncSetAttribute(fft::pow2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max));
  const int l2 = fft::log2_exact(n);
  if (l2 >= 0) {
    if (n > fft::kMaxPow2) return LIME_ERR_UNSUPPORTED;
    fft::Pass p{};
    p.n = n; p.log2n = l2; p.inverse = d->inverse;
    p.x = reinterpret_cast<const double2*>(d->x); p.x_s = d->x_s; p.x_bs = d->x_bs;
    p.y = reinterpret_cast<double2*>(d->y); p.y_s = d->y_s; p.y_bs = d->y_bs;
    p.shift = d->shift;
    p.post = reinterpret_cast<const double2*>(d->post);
    p.scale = 1.0;
    fft::pow2_kernel<<<d->batch, fft::kThreads, (size_t)n * sizeof(double2), st>>>(p);
    LIME_CUDA_TRY(cudaGetLastError());
    count_launch();
    return LIME_OK;
  }
  const int m = fft::bluestein_len(n);
  if (m > fft::kMaxPow2) return LIME_ERR_UNSUPPORTED;
  if (!d->workspace || d->workspace_bytes < lime_fft_f64_workspace(n, d->batch)) return LIME_ERR_WORKSPACE;
  double2* a = reinterpret_cast<double2*>(d->workspace);     // [batch][m]
  double2* f = a + (size_t)d->batch * m;                      // [m]
  const int lm = fft::log2_exact(m);
  const int64_t tot = (int64_t)d->batch * m;
  const int gb = (int)((tot + 255) / 256 < 65535 ? (tot + 255) / 256 : 65535);
  fft::chirp_in_kernel<<<gb, 256, 0, st>>>(reinterpret_cast<const double2*>(d->x), d->x_s, d->x_bs, n, m, d->batch,
                                           sgn, a);
  LIME_CUDA_TRY(cudaGetLastError());
  fft::chirp_filter_kernel<<<(m + 255) / 256, 256, 0, st>>>(n, m, sgn, f);
  LIME_CUDA_TRY(cudaGetLastError());
  fft::Pass p{};
  p.n = m; p.log2n = lm; p.scale = 1.0;
  // F = FFT(filter), in place
  p.inverse = 0; p.x = f; p.x_s = 1; p.x_bs = m; p.y = f; p.y_s = 1; p.y_bs = m;
  fft::pow2_kernel<<<1, fft::kThreads, (size_t)m * sizeof(double2), st>>>(p);
  LIME_CUDA_TRY(cudaGetLastError());
  // A = FFT(a) * F, in place
  p.x = a; p.y = a; p.mul = f;
  fft::pow2_kernel<<<d->batch, fft::kThreads, (size_t)m * sizeof(double2), st>>>(p);
  LIME_CUDA_TRY(cudaGetLastError());
  // conv = IFFT(A) (unscaled), in place
  p.inverse = 1; p.mul = nullptr;
  fft::pow2_kernel<<<d->batch, fft::kThreads, (size_t)m * sizeof(double2), st>>>(p);
  LIME_CUDA_TRY(cudaGetLastError());
  const int64_t tn = (int64_t)d->batch * n;
  const int go = (int)((tn + 255) / 256 < 65535 ? (tn + 255) / 256 : 65535);
  fft::chirp_out_kernel<<<go, 256, 0, st>>>(a, n, m, d->batch, sgn, d->shift,
                                            reinterpret_cast<const double2*>(d->post),
                                            reinterpret_cast<double2*>(d->y), d->y_s, d->y_bs);
  LIME_CUDA_TRY(cudaGetLastError());
  count_launch(6);
  return LIME_OK;
}
