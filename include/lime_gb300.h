/*
 * lime_gb300 — C ABI of the GB300 (sm_103a) open-system density-matrix
 * propagator.
 *
 * The reference (binggu56/lime) is pure Python and has no FFI; each entry
 * point below replaces the inner loop of one reference solver and is bound
 * from Python through ctypes (lime_gb300/_native.py).  Conventions:
 *
 *  - Complex matrices are interleaved (re, im) pairs, row-major,
 *    instance-major: element (b, i, j) of a [B][N][N] array sits at
 *    ((b * stride) + i * N + j) complex elements from the base, where
 *    ``stride`` is the per-instance stride in complex elements (0 = one
 *    matrix shared by every instance).
 *  - All pointers are DEVICE pointers owned by the caller.  No entry point
 *    allocates, frees or synchronises; work is enqueued on ``stream``.
 *  - Every entry point returns LIME_OK (0) or a negative lime_status and
 *    never throws.  Errors found by a kernel (non-finite values, trace
 *    drift) are written to the caller's device ``status`` word as a
 *    bit mask (LIME_FLAG_*) and read by the caller after the stream syncs.
 *  - Calls on different streams with disjoint buffers are independent.
 *
 * Physics: every propagator integrates the Lindblad generator written as
 *     d rho/dt = -i (Heff rho - rho Heff^dag) + sum_k L_k rho L_k^dag
 *     Heff     = H - (i/2) sum_k L_k^dag L_k
 * (algebraically identical to -i[H, rho] + sum_k (L rho L^dag - 1/2{L^dag L, rho}),
 * lime/oqs.py:706-723), with classic RK4 steps (lime/phys.py:636-649).
 * Collapse operators that are diagonal (L_k = diag(l_k)) enter through the
 * Hermitian matrix M = sum_k l_k l_k^dag:  sum_k L_k rho L_k^dag = M o rho.
 * The propagators act on Hermitian rho; a non-Hermitian rho is propagated as
 * its two Hermitian parts (the generator is linear and Hermiticity-preserving).
 */
#ifndef LIME_GB300_H
#define LIME_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  LIME_OK = 0,
  LIME_ERR_ARG = -1,          /* bad size, stride, pointer or alignment     */
  LIME_ERR_UNSUPPORTED = -2,  /* valid request this build does not handle  */
  LIME_ERR_CUDA = -3,         /* a CUDA runtime call failed                */
  LIME_ERR_NO_DEVICE = -4,    /* no sm_103 device current                  */
  LIME_ERR_WORKSPACE = -5,    /* workspace too small                       */
  LIME_ERR_SCRATCH_LIMIT = -6,/* request needs more than the fixed scratch  */
                              /* of lime_lindblad_rk4_f64_noalloc           */
} lime_status;

/* bits of the device status word written by kernels */
#define LIME_FLAG_NONFINITE   0x1  /* a NaN/Inf appeared in rho            */
#define LIME_FLAG_TRACE_DRIFT 0x2  /* |Tr rho(t) - Tr rho(0)| > trace_tol   */
#define LIME_FLAG_TIMEOUT     0x4  /* a bounded device-side wait expired    */
#define LIME_FLAG_RANGE       0x8  /* a split-precision operand left its    */
                                   /* fixed-point range (rescale and rerun) */
#define LIME_FLAG_NOT_HERMITIAN 0x10 /* rho(0) is not Hermitian: the batched */
                                   /* split kernel's results are invalid;   */
                                   /* run its two Hermitian parts instead   */
#define LIME_FLAG_BOUNDS      0x20 /* bounds-checked build (LIME_CHECK)    */
                                   /* only: an index left its buffer; the   */
                                   /* access was skipped                    */

/* ------------------------------------------------------------------ */
/* Generator preparation                                               */
/* ------------------------------------------------------------------ */

/* Build Heff = H - (i/2) sum_k L_k^dag L_k  and  M = sum_k l_k l_k^dag.
 * Replaces the per-RHS products dag(l).dot(l) of lime/oqs.py:716-723.
 *   h         [B|1][n][n] complex128, stride h_stride (0 = shared)
 *   l_dense   [B|1][k_dense][n][n] complex128 dense collapse ops, or NULL
 *   l_diag    [B|1][k_diag][n]     complex128 diagonals of diagonal ops, or NULL
 *   heff      [B][n][n] complex128 out
 *   m         [B][n][n] complex128 out (zero without diagonal operators)
 *   dephasing [B|1][n] float64 site-dephasing rates r_k, or NULL: the n
 *             operators sqrt(r_k)|k><k| given by their rates, which add
 *             r_k to the k-th diagonal entry of sum_k L_k^dag L_k and of M;
 *             stride dephasing_stride (0 = shared)
 */
typedef struct {
  int32_t n, batch, k_dense, k_diag;
  const double* h;        int64_t h_stride;
  const double* l_dense;  int64_t l_dense_stride;
  const double* l_diag;   int64_t l_diag_stride;
  double* heff;
  double* m;
  const double* dephasing; int64_t dephasing_stride;
} LimePrepareDesc;

int lime_lindblad_prepare_f64(const LimePrepareDesc* d, void* stream);

/* ------------------------------------------------------------------ */
/* Plain FP64 Lindblad RK4                                              */
/* ------------------------------------------------------------------ */

/* RK4 propagation of B Hermitian density matrices in FP64.
 * Replaces the time loop of _lindblad (lime/oqs.py:1590-1688) and
 * _correlation_2p_1t (lime/oqs.py:726-800):
 *   rho       [B][n][n] in: rho(t0); out: rho(t0 + n_steps dt)
 *   param_batch P: instance b uses parameter set p = b % P for heff, m,
 *             l_dense and obs_ops (0 means P = B).  A non-Hermitian input
 *             split into its Hermitian parts runs as B = 2P instances.
 *   heff      [P|1][n][n]           (from lime_lindblad_prepare_f64)
 *   m         [P|1][n][n] or NULL   (diagonal collapse operators)
 *   l_dense   [P|1][k_dense][n][n] or NULL
 *   obs_ops   [P|1][n_obs][n][n] observables (obs_diag = 0), or their
 *             diagonals [P|1][n_obs][n] when every observable is diagonal
 *             (obs_diag = 1), stride obs_stride per parameter set (0 =
 *             shared); obs_out[B][n_steps / obs_every][n_obs] receives
 *             Tr(E rho) after steps obs_every-1, 2*obs_every-1, ...
 *             (obs_every = 1: after every step, t = (k+1) dt, the
 *             reference's Result.observables timing, lime/oqs.py:1674-1682)
 *   states    [B][n_steps / states_every][n][n] or NULL: rho after steps
 *             states_every-1, 2*states_every-1, ...
 *   workspace caller-allocated, lime_lindblad_rk4_f64_workspace() bytes
 *   status    one int32 on the device (OR-ed LIME_FLAG_* bits)
 *   trace_tol trace-drift bound (<= 0 disables the check)
 */
typedef struct {
  int32_t n, batch, param_batch, n_steps, k_dense, n_obs, obs_diag, obs_every, states_every;
  double dt, trace_tol;
  double* rho;
  const double* heff;     int64_t heff_stride;
  const double* m;        int64_t m_stride;
  const double* l_dense;  int64_t l_dense_stride;
  const double* obs_ops;  int64_t obs_stride;
  double* obs_out;
  double* states;
  void* workspace;        size_t workspace_bytes;
  int32_t* status;
  /* time-dependent Hamiltonian H(t) = H0 - sum_q f_q(t) H_q (the driven
   * solver, lime/oqs.py:1691-1800): drive_ops [n_drive][n][n] complex128
   * Hermitian, drive_coef [n_steps][n_drive] real f_q(t0 + (k+1) dt) for
   * step k of this call.  n_drive = 0 for a static generator. */
  int32_t n_drive;
  const double* drive_ops;
  const double* drive_coef;
} LimeLindbladDesc;

size_t lime_lindblad_rk4_f64_workspace(int32_t n, int32_t batch, int32_t k_dense);
int lime_lindblad_rk4_f64(const LimeLindbladDesc* d, void* stream);

/* ------------------------------------------------------------------ */
/* Discrete adjoint (gradients) of the FP64 Lindblad RK4 path           */
/* ------------------------------------------------------------------ */

/* Backpropagates one checkpoint segment of steps [step0, step0 + seg_steps)
 * through the RK4 steps of lime_lindblad_rk4_f64 (no counterpart in the
 * reference, which has no gradients).  Per instance (one CTA):
 *   1. recompute rho_{step0..step0+seg_steps-1} from the checkpoint
 *      ckpt = rho_{step0};
 *   2. walking the steps backwards, add the observable source
 *      Herm(g E^dag) for every observable recorded after the step
 *      (obs_grad[B][total_steps/obs_every][n_obs] = dL/d conj(obs), torch's
 *      complex-gradient convention), recompute the stage states and apply
 *      the exact adjoint of the RK4 step with the adjoint generator
 *      L^dag(x) = -i(Ga x - x Ga^dag) + Madj o x + sum_k Ladj_k x Ladj_k^dag
 *      (Ga = -Heff^dag, Madj = conj(M), Ladj_k = L_k^dag);
 *   3. accumulate dL/dH_kk (grad_diag[B][n]), dL/dH_{k,k+1} for a real
 *      symmetric bond (grad_bond[B][n-1]) and dL/dgamma_k for dephasing
 *      operators sqrt(gamma_k)|k><k| (grad_gamma[B][n]) over the stages.
 * lam [B][n][n]: in, the adjoint state at step0 + seg_steps; out, at step0.
 */
typedef struct {
  int32_t n, batch, param_batch, seg_steps, step0, total_steps;
  int32_t k_dense, n_obs, obs_diag, obs_every;
  double dt;
  const double* ckpt;
  double* lam;
  const double* heff;       int64_t heff_stride;
  const double* m;          int64_t m_stride;
  const double* l_dense;    int64_t l_dense_stride;
  const double* heff_adj;   int64_t heff_adj_stride;
  const double* m_adj;      int64_t m_adj_stride;
  const double* l_dense_adj; int64_t l_dense_adj_stride;
  const double* obs_ops;    int64_t obs_stride;
  const double* obs_grad;
  double* grad_diag;
  double* grad_bond;
  double* grad_gamma;
  void* workspace;          size_t workspace_bytes;
} LimeAdjointDesc;

size_t lime_lindblad_adjoint_f64_workspace(int32_t n, int32_t batch, int32_t seg_steps, int32_t k_dense);
int lime_lindblad_adjoint_f64(const LimeAdjointDesc* d, void* stream);

/* ------------------------------------------------------------------ */
/* Bloch-Redfield generator and FP64 RK4 on vec(rho)                    */
/* ------------------------------------------------------------------ */

/* Dense Redfield generator in the eigenbasis of H, row-major Liouville
 * index a*n+b.  Replaces the N^2 K spectral-density loop and the sparse kron
 * products of redfield_tensor (lime/oqs.py:528-579); eigh, the eigenbasis
 * transform A_k = V^dag a_k V and the (user callback) spectra stay with the
 * caller, as in the reference.
 *   evals  [n] eigenvalues E
 *   a_eig  [k][n][n] complex128, A_k in the eigenbasis
 *   spec   [k|1][n][n] real, C_k[n][m] = S_k(-(E_n - E_m)); spec_stride = 0
 *          shares one matrix between all k
 *   R      [n^2][n^2] complex128 out: d vec(rho)/dt = R vec(rho)
 */
typedef struct {
  int32_t n, k;
  const double* evals;
  const double* a_eig;
  const double* spec;     int64_t spec_stride;
  double* R;
  void* workspace;        size_t workspace_bytes;
} LimeRedfieldBuildDesc;

size_t lime_redfield_build_f64_workspace(int32_t n, int32_t k);
int lime_redfield_build_f64(const LimeRedfieldBuildDesc* d, void* stream);

/* RK4 of a block of right-hand sides vec(rho_r) under a dense generator R in
 * FP64: replaces the time loop of _redfield (lime/oqs.py:453-462, rhs =
 * R.dot at 471-472).
 *   rho     [n^2][n_rhs] complex128 in/out (column r = row-major vec rho_r)
 *   obs_ops [n_obs][n][n] (eigenbasis); obs_out [n_steps/obs_every][n_rhs][n_obs]
 *           = Tr(E rho_r) after steps obs_every-1, 2*obs_every-1, ...
 *   states  [n_steps/states_every][n^2][n_rhs] or NULL
 */
typedef struct {
  int32_t n, n_rhs, n_steps, n_obs, obs_every, states_every;
  double dt;
  const double* R;
  double* rho;
  const double* obs_ops;
  double* obs_out;
  double* states;
  void* workspace;        size_t workspace_bytes;
} LimeRedfieldRK4Desc;

size_t lime_redfield_rk4_f64_workspace(int32_t n, int32_t n_rhs);
int lime_redfield_rk4_f64(const LimeRedfieldRK4Desc* d, void* stream);

/* The assembly step of lime_redfield_build_f64 alone, from caller-supplied
 * factors (for a differentiable generator whose factors the caller builds
 * and differentiates; replaces the same loop of redfield_tensor,
 * lime/oqs.py:528-579):
 *   evals [n]; a_eig, lam [k][n][n] complex128 with Lam_k = C_k o A_k;
 *   p, q [n][n] complex128: P = sum_k A_k Lam_k, Q = sum_k Lam_k^dag A_k;
 *   R [n^2][n^2] complex128 out (the closed form above). */
typedef struct {
  int32_t n, k;
  const double* evals;
  const double* a_eig;
  const double* lam;
  const double* p;
  const double* q;
  double* R;
} LimeRedfieldAssembleDesc;

int lime_redfield_assemble_f64(const LimeRedfieldAssembleDesc* d, void* stream);

/* Adjoint of lime_redfield_assemble_f64 (no counterpart in the reference,
 * which has no gradients): given G = dl/dconj(R) (the gradient of a real
 * loss l in the convention dl = Re sum conj(G) dR), writes the gradients of
 * the factors in the same convention: grad_evals [n] (real), grad_a and
 * grad_lam [k][n][n], grad_p and grad_q [n][n] (all complex128, overwritten).
 * The chain rule through Lam_k = C_k o A_k, P, Q, A_k = V^dag a_k V and
 * eigh(H) is the caller's (O(N^3 K) against the O(N^4 K) done here). */
typedef struct {
  int32_t n, k;
  const double* a_eig;
  const double* lam;
  const double* G;
  double* grad_evals;
  double* grad_a;
  double* grad_lam;
  double* grad_p;
  double* grad_q;
} LimeRedfieldAssembleAdjointDesc;

int lime_redfield_assemble_adjoint_f64(const LimeRedfieldAssembleAdjointDesc* d, void* stream);

/* Discrete adjoint of lime_redfield_rk4_f64 over one checkpoint segment of
 * seg_steps steps starting at step0 (no counterpart in the reference): the
 * segment is recomputed from ckpt storing every stage input y_i, then per
 * step from the last: lam += Et^dag g for the observables recorded after the
 * step (obs_grad [n_slots][n_rhs][n_obs] = dl/dconj(obs), laid out like
 * lime_redfield_rk4_f64's obs_out), the adjoint RK4 stages with L^dag
 * (a_4 = dt/6 lam, a_3 = dt/3 lam + dt L^dag a_4, a_2 = dt/3 lam +
 * dt/2 L^dag a_3, a_1 = dt/6 lam + dt/2 L^dag a_2, lam += sum_i L^dag a_i),
 * grad_R += sum_i a_i y_i^dag and grad_obs[o][j][i] += g_o conj(rho[i][j]).
 *   ckpt    [n^2][n_rhs] state at step0 (column r = vec rho_r)
 *   lam     [n^2][n_rhs] in: adjoint state after the segment; out: at step0
 *   grad_R  [n^2][n^2] accumulated; grad_obs [n_obs][n][n] accumulated or NULL
 *   workspace lime_redfield_adjoint_f64_workspace(n, n_rhs, seg_steps) bytes */
typedef struct {
  int32_t n, n_rhs, seg_steps, step0, n_obs, obs_every, n_slots;
  double dt;
  const double* R;
  const double* ckpt;
  double* lam;
  const double* obs_ops;
  const double* obs_grad;
  double* grad_R;
  double* grad_obs;
  void* workspace;        size_t workspace_bytes;
} LimeRedfieldAdjointDesc;

size_t lime_redfield_adjoint_f64_workspace(int32_t n, int32_t n_rhs, int32_t seg_steps);
int lime_redfield_adjoint_f64(const LimeRedfieldAdjointDesc* d, void* stream);

/* The same RK4 on the tcgen05 tensor cores in split precision: per stage
 * one GEMM [Yr|Yi] = [Lr|Li] . [[Sr,Si],[-Si,Sr]] with the operands streamed
 * by bulk copies from pre-tiled fp16 pieces (A = R, each row scaled by a
 * power of two and split into a 7-bit fixed-point part + two fp16
 * residuals; B = stage input: 10-bit fixed point + fp16 residual), exact
 * dominant product, fp32 two-sum accumulation, RK4 state in fp32 hi + lo.
 * Observables are a second GEMM of the same form (A = the observables,
 * K split across CTAs, fp64 partial sums).  Replaces the same loop as
 * lime_redfield_rk4_f64.
 *   R        [n^2][n^2] complex128 (from lime_redfield_build_f64)
 *   rho      [n_rhs][n^2] complex128 in/out, row-major vec(rho_r) per RHS
 *   scale_b_log2  rho * 2^b with max |rho(t)| * 2^b <= 2^13 at all times
 *            (2^13 / (1.25 max |rho0|) for trace-preserving generators);
 *            a state leaving that range raises LIME_FLAG_RANGE
 *   obs_ops  [n_obs][n][n]; obs_out [n_steps/obs_every][n_rhs][n_obs]
 *            (<E_o> = Tr(E_o rho) after steps obs_every, 2 obs_every, ...)
 *   workspace lime_redfield_split_workspace(n, n_rhs, n_obs) bytes,
 *            1024-byte aligned
 *   status   device int32 (LIME_FLAG_* bits)
 *   stage_out  NULL, or fp32 [4 n_steps + 1][2 Rp][Dp] (Rp = n_rhs rounded
 *            up to 64, Dp = n^2 rounded up to 128): every stage input of
 *            the call and the final state, component-planar, in the layout
 *            lime_redfield_adjoint_split takes as stage_in (the block form
 *            only; lime_redfield_rk4_split3 rejects it)
 */
typedef struct {
  int32_t n, n_rhs, n_steps, n_obs, obs_every;
  int32_t scale_b_log2;
  double dt;
  const double* R;
  double* rho;
  const double* obs_ops;
  double* obs_out;
  void* workspace;        size_t workspace_bytes;
  int32_t* status;
  float* stage_out;
} LimeRedfieldSplitDesc;

size_t lime_redfield_split_workspace(int32_t n, int32_t n_rhs, int32_t n_obs);
int lime_redfield_rk4_split(const LimeRedfieldSplitDesc* d, void* stream);

/* The same propagation with the complex product in its 3M form: per stage
 * the three real products T1 = Lr Sr, T2 = Li Si, T3 = (Lr + Li)(Sr + Si)
 * (one streaming launch over all three; Yr = T1 - T2, Yi = T3 - T1 - T2
 * formed from their fp32 two-sum words in an elementwise stage kernel with
 * the RK4 update), three quarters of the tensor-core products of the block
 * form.  Same descriptor and semantics as lime_redfield_rk4_split (the sum
 * operand Sr + Si is held at half the state scale); workspace
 * lime_redfield_split3_workspace(n, n_rhs, n_obs) bytes, 1024-byte aligned. */
size_t lime_redfield_split3_workspace(int32_t n, int32_t n_rhs, int32_t n_obs);
int lime_redfield_rk4_split3(const LimeRedfieldSplitDesc* d, void* stream);

/* The discrete adjoint of lime_redfield_rk4_split over one checkpoint
 * segment, on the tensor cores (no counterpart in the reference): the
 * recursion of lime_redfield_adjoint_f64 with every generator application
 * a streaming split-precision GEMM — the segment recomputed from ckpt with
 * L, the adjoint stages with L^dag (a_i scaled per step by the power of two
 * that maps (dt/2) max |lam| to 2^13 / 1.25 / 2^margin_log2), and the
 * generator gradient sum_i a_i y_i^dag of each step as one GEMM of K = four
 * stages x right-hand sides into an fp32 two-sum accumulator, added to
 * grad_R at the end of the call.
 *   ckpt, lam   [n_rhs][n^2] complex128 (row-major vec per right-hand side,
 *               as lime_redfield_rk4_split's rho); lam in/out
 *   scale_b_log2  the state scale of lime_redfield_rk4_split
 *   obs_ops, obs_grad, grad_R, grad_obs as in lime_redfield_adjoint_f64
 *   status    device int32: LIME_FLAG_RANGE (repeat with a larger margin)
 *   workspace lime_redfield_adjoint_split_workspace(n, n_rhs, seg_steps,
 *             n_obs) bytes, 1024-byte aligned
 *   stage_in  NULL (recompute the segment from ckpt), or the segment's
 *             stage inputs as written by lime_redfield_rk4_split's stage_out
 *             when it propagated this segment from ckpt with the same
 *             scale_b_log2 (the recompute is skipped; same results) */
typedef struct {
  int32_t n, n_rhs, seg_steps, step0, n_obs, obs_every, n_slots;
  int32_t scale_b_log2, margin_log2;
  double dt;
  const double* R;
  const double* ckpt;
  double* lam;
  const double* obs_ops;
  const double* obs_grad;
  double* grad_R;
  double* grad_obs;
  void* workspace;        size_t workspace_bytes;
  int32_t* status;
  const float* stage_in;
} LimeRedfieldAdjointSplitDesc;

size_t lime_redfield_adjoint_split_workspace(int32_t n, int32_t n_rhs, int32_t seg_steps, int32_t n_obs);
int lime_redfield_adjoint_split(const LimeRedfieldAdjointSplitDesc* d, void* stream);

/* ------------------------------------------------------------------ */
/* Green's-function route and basis changes (FP64)                      */
/* ------------------------------------------------------------------ */

/* Strided batched complex128 GEMM
 *     C[z][i][j] = sum_k op(A)[z][i][k] * scale[z][k] * op(B)[z][k][j]
 * for z < batch, i < M, j < N, k < K; op conjugates when conj_a / conj_b
 * is 1.  Strides are in complex elements (row, column, batch; 0
 * broadcasts); scale is optional (NULL: 1).  Replaces the propagator and
 * Green's-function contractions of Redfield_solver (lime/oqs.py:169-366:
 * U(t_z) = U1 diag(exp(w t_z)) U1^-1 as one call with scale = exp(w t_z),
 * expect, correlation_2op_1t, correlation_4op_3t) and the eigenbasis
 * transforms V^dag X V (lime/phys.py:706-718, lime/oqs.py:430-440). */
typedef struct {
  int32_t M, N, K, batch;
  int32_t conj_a, conj_b;
  const double* A;        int64_t a_rs, a_cs, a_bs;
  const double* B;        int64_t b_rs, b_cs, b_bs;
  const double* scale;    int64_t s_ks, s_bs;
  double* C;              int64_t c_rs, c_cs, c_bs;
} LimeZgemmDesc;

int lime_zgemm_strided_f64(const LimeZgemmDesc* d, void* stream);

/* Batched complex128 discrete Fourier transform along one axis:
 *     Y[b][k] = sum_j x[b][j] exp(-+ 2 pi i j k / n)    (- forward, + inverse;
 *                                                       no 1/n)
 * written to position (k + n/2) % n when shift = 1 (numpy's fftshift) and
 * multiplied there by post[position] when post is not NULL.  With post =
 * dx exp(-i w x0) this is lime's fft (lime/fft.py:9-56).  Strides in
 * complex elements (along the transform, between transforms).  Power-of-two
 * n <= 8192 need no workspace; other n <= 4096 take
 * lime_fft_f64_workspace(n, batch) bytes (16-byte aligned);
 * LIME_ERR_UNSUPPORTED above. */
typedef struct {
  int32_t n, batch, inverse, shift;
  const double* x;        int64_t x_s, x_bs;
  double* y;              int64_t y_s, y_bs;
  const double* post;
  void* workspace;        size_t workspace_bytes;
} LimeFftDesc;

size_t lime_fft_f64_workspace(int32_t n, int32_t batch);
int lime_fft_f64(const LimeFftDesc* d, void* stream);

/* ------------------------------------------------------------------ */
/* General Lindblad RK4 on the tensor cores (split precision)           */
/* ------------------------------------------------------------------ */

/* Any dimension, dense collapse operators: per RK4 stage two streaming
 * tcgen05 GEMMs per instance, [X; Y_1..Y_K] = [Heff; L_1..L_K] rho_s and
 * Z = [L_1 | .. | L_K] [Y_1^dag; ..; Y_K^dag] = sum_k L_k rho_s L_k^dag,
 * with the split-precision operands of lime_redfield_rk4_split, then
 * f = Z - i(X - X^dag) + M o rho_s and the RK4 update fused into the second
 * GEMM's epilogue.  Replaces the same loops as lime_lindblad_rk4_f64 for
 * Hermitian rho (run a non-Hermitian start as its two Hermitian parts).
 *   rho       [B][n][n] complex128 in/out
 *   heff      [P|1][n][n] (lime_lindblad_prepare_f64), stride heff_stride
 *   m         [P|1][n][n] or NULL (diagonal collapse operators), m_stride
 *   l_ops     [P|1][n_ops][n][n] dense collapse operators or NULL, l_stride
 *   obs_ops   [P|1][n_obs][n][n], obs_stride; obs_out [B][n_steps/obs_every][n_obs]
 *             Tr(E rho) after steps obs_every, 2 obs_every, ...
 *   scale_b_log2  rho * 2^b, max |rho(t)| 2^b <= 2^13
 *   scale_y_log2  (L_k rho) * 2^y, max |L_k rho(t)| 2^y <= 2^13
 *             (a value out of range raises LIME_FLAG_RANGE)
 *   workspace lime_lindblad_stream_workspace(n, batch, G, n_ops) bytes,
 *             1024-byte aligned; G = 1 when heff and l_ops are shared
 *             (strides 0), else param_batch
 */
typedef struct {
  int32_t n, batch, param_batch, n_ops, n_steps, n_obs, obs_every;
  int32_t scale_b_log2, scale_y_log2;
  double dt;
  double* rho;
  const double* heff;     int64_t heff_stride;
  const double* m;        int64_t m_stride;
  const double* l_ops;    int64_t l_stride;
  const double* obs_ops;  int64_t obs_stride;
  double* obs_out;
  void* workspace;        size_t workspace_bytes;
  int32_t* status;
  /* driven generator, as in LimeLindbladDesc: Heff(t) = Heff - sum_q
   * drive_coef[k][q] drive_ops[q] during step k (rebuilt and re-split on
   * the device every step); n_drive = 0 for a static generator */
  int32_t n_drive;
  const double* drive_ops;
  const double* drive_coef;
  /* a diagonal M (real M_ii, [P|1][n], stride n or 0) instead of m: the
   * jump term then touches only the diagonal (pure dephasing) */
  const double* m_diag;   int64_t m_diag_stride;
  /* 1: obs_ops holds only the diagonals of diagonal observables,
   * [P|1][n_obs][n] complex128 (obs_stride n_obs n or 0), and
   * Tr(E rho) = sum_x E_xx rho_xx reads n state elements */
  int32_t obs_diag;
} LimeLindbladStreamDesc;

size_t lime_lindblad_stream_workspace(int32_t n, int32_t batch, int32_t n_generators, int32_t n_ops);
int lime_lindblad_rk4_stream(const LimeLindbladStreamDesc* d, void* stream);

/* An uneven batch: n_groups propagations of the form above (each its own
 * dimension, operator count, batch, buffers, workspace and status word)
 * with a common n_steps, dt and obs_every and no drive, run in lockstep:
 * per RK4 stage ONE persistent launch runs the GEMM 1 tiles of every group
 * and one the GEMM 2 tiles (a CTA per SM loops over the concatenated tile
 * list, starting the next tile's operand copies and MMAs while the epilogue
 * of the previous one runs).  Replaces the per-instance calls of
 * lime/oqs.py:1590-1688 for instances of different sizes.
 *   n_ctas    persistent CTAs per launch (0: one per SM)
 *   order     1: tiles of the groups with the most K chunks per tile first
 *             (longest first); 0: groups in the given order
 * Returns LIME_ERR_UNSUPPORTED for n_groups > lime_lindblad_stream_max_groups()
 * or a driven group.  Range retries are per group, through
 * lime_lindblad_rk4_stream. */
int32_t lime_lindblad_stream_max_groups(void);
int lime_lindblad_rk4_stream_groups(const LimeLindbladStreamDesc* descs, int32_t n_groups, int32_t n_ctas,
                                    int32_t order, void* stream);

/* Discrete adjoint of the RK4 steps of lime_lindblad_rk4_stream for the
 * chain model (site energies on the diagonal, nearest-neighbour bonds, site
 * dephasing; no dense collapse operators): the same backward recursion and
 * gradient sums as lime_lindblad_adjoint_f64, over all segments in one
 * call, on the tensor cores.  Per segment (from the last): recompute the
 * forward steps from the checkpoint, storing every stage input, then walk
 * the steps backwards applying the adjoint generator (G = -Heff^dag, conj M)
 * through the same streaming GEMM.
 *   ckpt      [n_seg][B][n][n] complex128: the state at steps 0, seg, 2 seg, ...
 *   lam       [B][n][n] complex128 out (adjoint state at step 0) or NULL
 *   heff, heff_adj = -Heff^dag  [P|1][n][n]; m, m_adj = conj(M) or both NULL
 *   obs_ops   [P|1][n_obs][n][n]; obs_grad [B][n_steps/obs_every][n_obs]
 *             complex128 = dL/d conj(obs) (torch's convention)
 *   grad_diag [B][n], grad_bond [B][max(n-1,1)], grad_gamma [B][n] (added to)
 *   scale_b_log2  power-of-two scale of rho (max |rho| 2^s <= 2^13); the
 *             adjoint stage inputs are scaled per step from max |lam| on the
 *             device (LIME_FLAG_RANGE if a value leaves the range)
 *   scale_l_log2  reserved (0)
 *   workspace lime_lindblad_adjoint_stream_workspace(n, batch, G, seg_steps),
 *             1024-byte aligned; G = 1 when heff and heff_adj are shared
 */
typedef struct {
  int32_t n, batch, param_batch, n_steps, seg_steps, n_obs, obs_every;
  int32_t scale_b_log2, scale_l_log2;
  double dt;
  const double* ckpt;
  double* lam;
  const double* heff;      int64_t heff_stride;
  const double* heff_adj;  int64_t heff_adj_stride;
  const double* m;
  const double* m_adj;     int64_t m_stride;
  const double* obs_ops;   int64_t obs_stride;
  const double* obs_grad;
  double* grad_diag;
  double* grad_bond;
  double* grad_gamma;
  void* workspace;         size_t workspace_bytes;
  int32_t* status;
  const double* m_diag;    int64_t m_diag_stride;   /* as in LimeLindbladStreamDesc (replaces m and m_adj) */
  /* optional: the observable sources' coefficients in fp32, float pairs
   * [P|1][n_obs][2][n][n] (same instance stride rule as obs_ops): for
   * component c of element (row, x), (Re E_xr + Re E_rx, Im E_xr + Im E_rx) / 2
   * (c = 0) and (Im E_rx - Im E_xr, Re E_xr - Re E_rx) / 2 (c = 1), so the
   * source is Re g Q.x + Im g Q.y; NULL: formed from obs_ops in FP64 */
  const float* obs_coef;
} LimeLindbladAdjointStreamDesc;

size_t lime_lindblad_adjoint_stream_workspace(int32_t n, int32_t batch, int32_t n_generators, int32_t seg_steps);
int lime_lindblad_adjoint_stream(const LimeLindbladAdjointStreamDesc* d, void* stream);

/* Same propagation as lime_lindblad_rk4_f64 for callers that cannot allocate
 * device memory: a host framework whose pool owns the GPU, a latency-critical
 * loop where cudaMalloc/cudaFree would synchronise the device, or a process
 * that must keep a fixed device footprint after start-up.  No counterpart in
 * the reference (which has no native code); it has no workspace argument:
 * d->workspace and d->workspace_bytes are ignored.
 *   - Scratch is a fixed LIME_NOALLOC_SCRATCH_BYTES array inside the
 *     library's device image, held on every GPU that loads the library until
 *     the process exits.  Requests whose workspace
 *     (lime_lindblad_rk4_f64_workspace) exceeds it return
 *     LIME_ERR_SCRATCH_LIMIT without launching anything.
 *   - The first call in each CUDA context looks up the array's device
 *     address (cudaGetSymbolAddress) with that context's device current;
 *     make that first call before any stream capture on the device.  A new
 *     context on the same device (after cudaDeviceReset, or another context
 *     the caller makes current) is recognised by its ID and looked up again,
 *     so that first call too belongs before any capture.
 *   - Nothing is allocated or freed by this call.
 *   - All calls in the process share one array per device and it keeps the
 *     previous call's contents; every word a call reads it first writes, but
 *     calls whose executions overlap on the GPU (different streams, or
 *     concurrent host threads) race on it and must be serialised by the
 *     caller.
 */
#define LIME_NOALLOC_SCRATCH_BYTES ((size_t)16 << 20)
size_t lime_noalloc_scratch_bytes(void);
int lime_lindblad_rk4_f64_noalloc(const LimeLindbladDesc* d, void* stream);

/* ------------------------------------------------------------------ */
/* Batched split-precision Lindblad RK4 (tensor cores)                  */
/* ------------------------------------------------------------------ */

/* RK4 propagation of B Hermitian density matrices (n <= 64) on the tcgen05
 * tensor cores: each stage's Heff * rho is a split-precision product (A:
 * per-row 7-bit fixed point + two fp16 residuals, B: per-row 10-bit fixed
 * point + fp16 residual, exact dominant product) of power-of-two pre-scaled
 * operands; the
 * state is fp32 with an fp32 compensation term; observables, traces and the
 * final state are produced in FP64.  Replaces the same loops as
 * lime_lindblad_rk4_f64 (lime/oqs.py:1674-1682, 777-787) for generators
 * whose collapse operators are site-diagonal projectors or any diagonal
 * operators with diagonal M (pure dephasing): m_diag[p][i] = M_ii.
 *   scale_a_log2  A = Heff * 2^scale_a_log2 (choose max|A| ~ 2^12)
 *   scale_b_log2  B = rho  * 2^scale_b_log2 (choose a bound of |rho_ij| ~ 2^13;
 *                 each B row then gets its own fixed-point quantum from the
 *                 previous stage's row bound)
 *   obs_mode      0 none; 1 populations: obs k = rho_kk (n_obs <= n);
 *                 2 dense: obs_ops [P|1][n_obs][n][n], Tr(E rho)
 *   obs_out       [B][n_steps / obs_every][n_obs] complex128
 *   ctas_per_sm   0 = default (2)
 *   n_drive       0, or the number of drive operators: the generator of step
 *                 k is Heff - sum_d drive_coef[k][d] drive_ops[d] (the
 *                 driven equation of lime/oqs.py:1691-1800, coefficients at
 *                 the end of the step, held through its four stages)
 *   drive_ops     [n_drive][n][n] complex128, shared by all instances
 *   drive_coef    [n_steps][n_drive] real
 *   workspace     n_drive > 0: lime_lindblad_split_workspace(n, param_batch,
 *                 n_drive, n_steps) bytes, 256-byte aligned (fp32 pair
 *                 copies of Heff, the drive operators and coefficients);
 *                 scale_a_log2 must cover max_k |Heff - sum_d c_d(k) mu_d|
 * Without a drive no workspace: state lives on chip for the whole launch.
 */
typedef struct {
  int32_t n, batch, param_batch, n_steps;
  int32_t obs_mode, n_obs, obs_every;
  int32_t scale_a_log2, scale_b_log2, ctas_per_sm;
  double dt, trace_tol;
  double* rho;
  const double* heff;     int64_t heff_stride;
  const double* m_diag;   int64_t m_stride;
  const double* obs_ops;  int64_t obs_stride;
  double* obs_out;
  int32_t* status;
  int32_t n_drive;
  const double* drive_ops;
  const double* drive_coef;
  void* workspace;        size_t workspace_bytes;
  /* optional (zero / NULL keeps the behaviour above):
   * a_pieces      the A operand prepared once per generator by
   *               lime_lindblad_split_prepare with the same heff and
   *               scale_a_log2 (undriven calls only); a_stride its bytes per
   *               parameter set (0 = shared, else 98304)
   * rho_out       [B][n][n] final state (NULL: written over rho)
   * auto_scale_b  1: each instance takes its B scale from its own rho(0),
   *               2^b sqrt(n) ||rho(0)||_F <= 2^13 (scale_b_log2 ignored)
   * chunk_steps   RK4 steps per launch (0: about 2^22 instance-steps per
   *               launch), rounded up to a multiple of obs_every; each
   *               launch continues from the state the previous one wrote
   *               to rho_out
   * Every instance's rho(0) is checked for Hermiticity on the float pair of
   * each element; a non-Hermitian one raises LIME_FLAG_NOT_HERMITIAN. */
  const void* a_pieces;   int64_t a_stride;
  double* rho_out;
  int32_t auto_scale_b;
  int32_t chunk_steps;
} LimeLindbladSplitDesc;

size_t lime_lindblad_split_workspace(int32_t n, int32_t param_batch, int32_t n_drive, int32_t n_steps);
int lime_lindblad_rk4_split(const LimeLindbladSplitDesc* d, void* stream);

/* The A operand of lime_lindblad_rk4_split, split once per generator instead
 * of once per instance and call (no reference counterpart: it hoists the
 * per-call operand conversion out of the time loop of lime/oqs.py:1590-1688):
 * each block row of 2^scale_a_log2 [[Hr, -Hi], [Hi, Hr]] as a per-row 7-bit
 * fixed-point part + two fp16 residuals, in the order the kernel stores them
 * to tensor memory.  heff [count][n][n] (stride heff_stride complex elements,
 * 0 with count 1); out: lime_lindblad_split_prepared_bytes(n, count) bytes,
 * 16-byte aligned. */
typedef struct {
  int32_t n, count, scale_a_log2;
  const double* heff;     int64_t heff_stride;
  void* out;              size_t out_bytes;
} LimeLindbladSplitPrepareDesc;

size_t lime_lindblad_split_prepared_bytes(int32_t n, int32_t count);
int lime_lindblad_split_prepare(const LimeLindbladSplitPrepareDesc* d, void* stream);

/* ------------------------------------------------------------------ */
/* Self-test of the bounded device-side waits (test infrastructure)     */
/* ------------------------------------------------------------------ */
/* Every device-side wait of the entry points above polls an mbarrier at most
 * a bounded number of times; on expiry the kernel ORs LIME_FLAG_TIMEOUT
 * into its status word, releases its tensor memory and returns (the C
 * ABI's "wait timeout" status; the context stays usable).  This entry point
 * makes such waits expire on purpose, with max_wait polls:
 *   kind 0  one CTA waits on an mbarrier that nothing completes  -> TIMEOUT
 *   kind 1  the same barrier, completed first (control)          -> 0
 *   kind 2  the streaming split-precision GEMM tile of the Redfield and
 *           general Lindblad paths with its operand copies withheld: the
 *           MMA and epilogue waits expire, the tile aborts      -> TIMEOUT
 *   kind 3  the same tile with its copies issued (control)       -> 0
 *   kind 4  bounds-checked build (liblime_gb300_check.so) only: the
 *           same tile told that its A operand holds one piece fewer than
 *           it reads; the producer's extent check refuses that copy, so
 *           nothing is read past the buffer, and the tile aborts
 *                                          -> LIME_FLAG_BOUNDS | TIMEOUT
 *           (the regular build returns LIME_ERR_UNSUPPORTED)
 * ws (kinds 2, 3; 16-byte aligned): lime_wait_selftest_workspace() bytes =
 * 10 zero operand pieces of 16 KB followed by 128 float row scales (1.0);
 * the control checks that the tile of zero operands comes out zero
 * (LIME_FLAG_NONFINITE otherwise).  status: device int32. */
size_t lime_wait_selftest_workspace(void);
int lime_wait_selftest(int kind, uint32_t max_wait, const void* ws, int32_t* status, void* stream);

/* ------------------------------------------------------------------ */
/* Library info                                                         */
/* ------------------------------------------------------------------ */

/* 0 when a device of compute capability 10.3 is current, else negative. */
int lime_device_check(void);
/* Cumulative number of kernels this library has enqueued (all entry points,
 * all threads); lets a caller count the launches inside a timed region. */
int64_t lime_launch_count(void);
const char* lime_status_string(int status);
int lime_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LIME_GB300_H */
