/*
 * ddcsvd.h -- C ABI of libddcsvd.so, a GB300 (sm_103a) implementation of the
 * ddc-svd dense SVD pipeline.
 *
 * Drop-in entry points keep the reference's signatures and argument layout:
 *   svd_gpu     replaces svd_gpu.h:5   (svd_gpu.c:53-131)
 *   bidiag_par  replaces bidiag_par.h:30 (bidiag_par.c:34-450)
 *   form_u_par, form_v_par  replace bidiag_par.h:33-34 (bidiag_par.c:877-988)
 * Everything else extends that interface (status codes, FP32 buffers, device
 * pointers, batching, the adjoint).  All matrices are column-major.  The
 * singular values come out ascending, as the reference returns them
 * (Calculations-Parallel.c:56); column i of U / V belongs to sigma[i].
 *
 * Errors: every int-returning function returns DDCSVD_OK (0) or one of the
 * DDCSVD_ERR_* codes; ddcsvd_last_error() gives a one-line description of the
 * last failure on the calling thread.  The void drop-ins cannot return a
 * status; on failure they fill sigma with NaN and print one line to stderr
 * (the reference aborts the process instead, svd_gpu.c:85).
 */
#ifndef DDCSVD_H
#define DDCSVD_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define DDCSVD_OK 0
#define DDCSVD_ERR_ARG 1       /* invalid size, stride or pointer            */
#define DDCSVD_ERR_CUDA 2      /* a CUDA runtime call failed                  */
#define DDCSVD_ERR_ALLOC 3     /* device or pinned host allocation failed     */
#define DDCSVD_ERR_NOCONV 4    /* an iteration hit its cap without converging */
#define DDCSVD_ERR_TIMEOUT 5   /* a device-side wait gave up (bounded spin)   */
#define DDCSVD_ERR_NODEVICE 6  /* no usable sm_103 device                     */
#define DDCSVD_ERR_NONFINITE 7 /* input holds NaN or Inf                      */
#define DDCSVD_ERR_UNSUPPORTED 8

/* ---------------------------------------------------------------- modes
 * Which bidiagonalisation / back-transformation the pipeline uses.
 *   PLAIN_FP32   unblocked Householder steps (rank-1 updates), reflectors
 *                applied one at a time -- the reference's algorithm shape on
 *                FP32 CUDA cores.
 *   BLOCKED_FP32 panel (WY / Bischof) bidiagonalisation with rank-2b trailing
 *                updates and WY back-transformation, FP32 CUDA-core GEMMs.
 *   BLOCKED_TF32X3 the same with the GEMMs on tcgen05 tensor cores in split
 *                TF32, two parts per operand (hi*hi + hi*lo + lo*hi, FP32
 *                accumulation in TMEM): about 21 bits per product.
 *   BLOCKED_BF16X3 reserved for split BF16 (returns DDCSVD_ERR_UNSUPPORTED).
 *   BLOCKED_TF32X6 split TF32 with three parts per operand and six products
 *                (h*h + h*m + m*h + m*m + h*l + l*h): FP32-level accuracy.
 *   AUTO         BLOCKED_TF32X6.                                           */
#define DDCSVD_MODE_AUTO 0
#define DDCSVD_MODE_PLAIN_FP32 1
#define DDCSVD_MODE_BLOCKED_FP32 2
#define DDCSVD_MODE_BLOCKED_TF32X3 3
#define DDCSVD_MODE_BLOCKED_BF16X3 4
#define DDCSVD_MODE_BLOCKED_TF32X6 5

typedef struct ddcsvd_context *ddcsvd_handle_t;

/* ---------------------------------------------------------------- drop-ins */

/* Replaces svd_gpu.h:5 / svd_gpu.c:53.  Host buffers, FP64 in and out.
 * The reference leaves A overwritten with its Householder reflectors
 * (bidiag_par.c:63-68); this implementation leaves A unchanged (callers of
 * the reference cannot rely on A after the call, and bidiag_par below still
 * returns the reflectors).  sigma: min(m,n) values, ascending.
 * U: m x min(m,n) (column i at U + i*m); V: n x min(m,n) (column i at V + i*n).
 * Computes in the default mode (DDCSVD_MODE env var, else AUTO): FP32
 * bidiagonalisation and back-transformation, FP64 singular values and
 * bidiagonal vectors. */
void svd_gpu(int m, int n, double *A, double *sigma, double *U, double *V);

/* Replaces bidiag_par.h:30 / bidiag_par.c:34.  Host buffers, any shape.
 * alpha: min(m,n) diagonal entries; beta: n-1 superdiagonal entries when
 * m >= n, m entries when m < n (the m x (m+1) upper bidiagonal of a wide
 * matrix, with the reference's last-row edge case, bidiag_par.c:361-383).  A is
 * overwritten with the reflectors as bidiag_par leaves it: the i-th left
 * reflector v in the partial column from A[i,i], the i-th right reflector in
 * the partial row from A[i,i+1], each with H = I - 2 v v^T and ||v|| = 1. */
void bidiag_par(int m, int n, double *A, double *alpha, double *beta);

/* Replace bidiag_par.h:33-34 (bidiag_par.c:877-988).  Host FP64 buffers.
 * From the reflectors that bidiag_par leaves in A_mod (m x n), form the full
 * left factor U (m x m, column i at U + i*m) or the right factor V (n x n),
 * so that A = U [B; 0] V^T; computed on the GPU in FP64 in the reference's
 * order.  On failure the first entry of the output is NaN and one line goes
 * to stderr (the reference has no error path). */
void form_u_par(int m, int n, const double *A_mod, double *U);
void form_v_par(int m, int n, const double *A_mod, double *V);

/* ---------------------------------------------------------------- status-returning host API */

/* svd_gpu with a status and an explicit mode (DDCSVD_MODE_*). */
int svd_gpu_ex(int m, int n, double *A, double *sigma, double *U, double *V, int mode);

/* FP32 host buffers, A is not modified.  lda >= m, ldu >= m, ldv >= n. */
int ddcsvd_svd_f32(int m, int n, const float *A, int lda, float *sigma, float *U, int ldu,
                   float *V, int ldv, int mode);
/* The same on a handle (its launch knobs, limits and stream; the call
 * returns after the results are in the host buffers). */
int ddcsvd_svd_f32_host(ddcsvd_handle_t handle, int m, int n, const float *A, int lda, float *sigma, float *U,
                        int ldu, float *V, int ldv, int mode);

/* ---------------------------------------------------------------- handles and device API */

/* A handle owns a CUDA stream, a device workspace, a stream-ordered memory
 * pool and pinned staging memory on one device.  Calls on one handle are serialised; use one handle per
 * host thread for concurrency.  device < 0 selects the current device. */
int ddcsvd_create(ddcsvd_handle_t *handle, int device);
int ddcsvd_destroy(ddcsvd_handle_t handle);
/* Work of this handle goes to `stream` (a cudaStream_t; NULL = the legacy default stream).
 * A new handle starts on a private non-blocking stream.  Part of an SVD in
 * the tensor-core modes runs on the handle's own second stream, forked from
 * and joined back to `stream` by events within the call. */
int ddcsvd_set_stream(ddcsvd_handle_t handle, void *stream);
/* Frees the cached device workspace and returns the memory that the
 * handle's own stream-ordered pool keeps between calls (per-call buffers of
 * the host API, the QR path and aligned output copies); both regrow on the
 * next call. */
int ddcsvd_release_workspace(ddcsvd_handle_t handle);

/* Full SVD, device pointers (FP32).  The call is asynchronous on the
 * handle's stream except that it reads back one status word at the end. */
int ddcsvd_svd_f32_device(ddcsvd_handle_t handle, int m, int n, const float *dA, int lda,
                          float *dSigma, float *dU, int ldu, float *dV, int ldv, int mode);

/* Stage 1 alone: FP32 bidiagonalisation of dA (m >= n) in place.  dA keeps
 * the reflectors in LAPACK form (unit leading entry implicit, scale in
 * dTauq / dTaup); dD (n) and dE (n-1) receive the bidiagonal. */
int ddcsvd_bidiag_f32_device(ddcsvd_handle_t handle, int m, int n, float *dA, int lda,
                             float *dD, float *dE, float *dTauq, float *dTaup, int mode);

/* Stage 2 alone (Calculations-Parallel.c:852 GetSingularValues_Parallel):
 * ascending singular values of the N x (N+1) upper bidiagonal with diagonal
 * dB1 (N) and superdiagonal dB2 (N; dB2[N-1] = 0 gives the square case). */
int ddcsvd_bdsdc_sigma_device(ddcsvd_handle_t handle, int N, const double *dB1, const double *dB2,
                              double *dSigma);

/* Stages 3-4 alone (parallel-twisted.c:554 CalcRightSingularVectors and :530
 * RighttoLeftSingularVectors): right (dX) and left (dY) singular vectors of
 * the N x N upper bidiagonal (dA diagonal N, dB superdiagonal N-1) for the
 * given ascending dSigma.  dX, dY: N x N column-major FP32, ld = N.  Values
 * that coincide to working precision inside one unreduced block (which the
 * reference's method maps to one repeated vector) get an orthonormal basis of
 * their common subspace. */
int ddcsvd_bdvec_device(ddcsvd_handle_t handle, int N, const double *dA, const double *dB,
                        const double *dSigma, float *dX, float *dY);

/* Host-only planning of stage 2 (no GPU work; for tests and tools).
 * ddcsvd_split_plan: splits the N x N bidiagonal a (N), b (N) at
 * |b_i| <= 4 eps max|entry| as the pipeline does (b_i set to 0 there, b[N-1]
 * too) and writes the block starts (ascending, first 0, last N; at most N+1)
 * to starts, their count to nstarts.
 * ddcsvd_dc_plan: the D&C forest the pipeline builds for those blocks
 * (Calculations-Parallel.c:706-850: node N splits at K = N/2 into K and
 * N-K-1, leaves N <= 2) and its schedule, as the packed int table uploaded
 * to the GPU: per node r0, n, slot, K, child1, child2 (nodes ordered by
 * depth), depth starts, merge starts, merge list, lanes per root by depth,
 * then per tree: tree segment starts, segment node starts, segment merge
 * ends, segment depths, segment lanes, nodes, trees by size.  meta[8] =
 * {nodes, max depth, merges, trees, segments, largest tree, offset of the
 * per-tree part, table length}; DDCSVD_ERR_ARG when cap is too small (meta
 * is filled either way). */
int ddcsvd_split_plan(int N, double *a, double *b, double eps, int *starts, int *nstarts);
int ddcsvd_dc_plan(int N, int nstarts, const int *starts, int terms_per_lane, int *out, long long cap, int *meta);

/* ---------------------------------------------------------------- batched */

/* Many independent SVDs of uneven sizes in one launch sequence (device
 * pointers).  Matrix b is dA + offA[b] (m[b] x n[b], column-major, ld m[b]);
 * its results go to dSigma + offS[b] (min(m,n)), dU + offU[b]
 * (m x min(m,n), ld m) and dV + offV[b] (n x min(m,n), ld n).  Offsets are
 * element offsets in host arrays. */
int ddcsvd_svd_batched_f32_device(ddcsvd_handle_t handle, int batch, const int *m, const int *n,
                                  const float *dA, const long long *offA, float *dSigma,
                                  const long long *offS, float *dU, const long long *offU,
                                  float *dV, const long long *offV);

/* ---------------------------------------------------------------- adjoint */

/* Reverse-mode derivative of the thin SVD A = U diag(s) V^T (m >= n, k = n)
 * for a batch of equally sized matrices (device pointers, FP64 or FP32 by
 * the _f64/_f32 suffix; strides between matrices are m*k, k, n*k, m*n).
 * Given dL/ds (gs), dL/dU (gU), dL/dV (gV) -- any may be NULL for zero --
 * writes dL/dA (gA, m x n):
 *   gA = U [diag(gs) + (F o (U^T gU - gU^T U)) S + S (F o (V^T gV - gV^T V))] V^T
 *        + (I - U U^T) gU S^-1 V^T,   F_ij = 1/(s_j^2 - s_i^2) (i != j), 0 on the diagonal.
 * The derivative does not exist where two singular values coincide
 * (s_i = s_j, i != j) or, with gU given, where one is zero: gA then holds
 * Inf or NaN and the status is still DDCSVD_OK.  Any batch size is accepted
 * (launches go in chunks of 65535 problems). */
int ddcsvd_svd_backward_f64_device(ddcsvd_handle_t handle, int batch, int m, int n,
                                   const double *dU, const double *dS, const double *dV,
                                   const double *gU, const double *gS, const double *gV,
                                   double *gA);
int ddcsvd_svd_backward_f32_device(ddcsvd_handle_t handle, int batch, int m, int n,
                                   const float *dU, const float *dS, const float *dV,
                                   const float *gU, const float *gS, const float *gV, float *gA);

/* No counterpart in the reference.  The FP64 adjoint above for callers that
 * must not allocate device memory when they call it -- code working inside
 * another framework's memory pool or a fixed, pre-planned memory budget, or a
 * latency-critical loop that must stay away from the driver's allocator.  It
 * takes no handle and calls no cudaMalloc / cudaFree / allocating library
 * routine: its intermediates live in a 16 MiB array compiled into this
 * library, which every GPU that loads the library holds until the process
 * exits.  Inputs and outputs are caller-owned device buffers (same layout as
 * ddcsvd_svd_backward_f64_device).  The call only enqueues its kernels on
 * `stream` (a cudaStream_t, NULL = legacy default stream) and returns; gA is
 * ready once that stream has been synchronised.  Launch-configuration errors
 * come back as DDCSVD_ERR_CUDA.  Limit: 3 r(8 batch n^2) + r(8 batch m n)
 * bytes, r(x) = x rounded up to a multiple of 256, must not exceed 16 MiB
 * (16777216), else DDCSVD_ERR_ARG (split the batch).  The first call in a
 * CUDA context looks up the array's device address in that context
 * (cudaGetSymbolAddress) and keeps it for the context's lifetime; make that
 * first call before any stream capture.  All calls share the one array:
 * calls whose GPU work overlaps (concurrent streams or threads) race and must
 * be serialised by the caller. */
int ddcsvd_svd_backward_f64_noalloc(void *stream, int batch, int m, int n, const double *dU,
                                    const double *dS, const double *dV, const double *gU,
                                    const double *gS, const double *gV, double *gA);

/* ---------------------------------------------------------------- autotuning */

/* No counterpart in the reference (the reference has no launch parameters).
 * Launch knobs of a handle, in this order:
 *   [0] split-K cap of the GEMMs (1 = never split, default 16)
 *   [1] tensor-core tile width (0 = by the output width, 64 = always 64)
 *   [2] batched stage-1 CTA size (256 or 512, default 512)
 *   [3] batched stage-1 residency (1 = whole problem in shared memory up to
 *       the SM's opt-in limit, default; 0 = up to 24K entries, two CTAs/SM)
 *   [4] D&C secular-sum terms per lane (2..32, default 8)
 *   [5] QR first for m >= 2n (or n >= 2m) in the tensor-core modes: 0 never,
 *       1 always, 2 (default) when the matrix has at least 64M entries
 *   [6] bidiagonalisation panels with at most 8192 rows: 1 (default) one
 *       read of the trailing block per column (y = A^T u and x = A v in one
 *       pass), 0 two separate products
 *   [7] bidiagonalisation tail: the last columns (at most this many,
 *       default 512; 0 never) run on one thread-block cluster with the
 *       trailing block in its shared memory (unblocked, no grid-wide
 *       barriers)
 * Knobs [0]-[4] and [6] change the results only through the summation order
 * of split-K, of the D&C sums and of the panel products; [5] and [7] change
 * the algorithm (equally accurate).
 * get/set copy up to `count` knobs. */
int ddcsvd_get_tuning(ddcsvd_handle_t handle, int *values, int count);
int ddcsvd_set_tuning(ddcsvd_handle_t handle, const int *values, int count);

/* Coordinate search over the knobs on seeded synthetic data of the given
 * single-matrix shape / batch of shapes (host arrays m, n), timed with CUDA
 * events on the handle's stream, `reps` timed runs per candidate; the
 * fastest values stay in the handle.  Allocates its own device buffers.
 * The single-matrix tuner covers knobs [0], [1] and (tall shapes) [5], the
 * batched tuner [2], [3] and [4]. */
int ddcsvd_autotune_svd(ddcsvd_handle_t handle, int m, int n, int mode, int reps);
int ddcsvd_autotune_batched(ddcsvd_handle_t handle, int batch, const int *m, const int *n, int reps);

/* ---------------------------------------------------------------- limits */

/* No counterpart in the reference, which has no error path: it aborts the
 * process on any failure (svd_gpu.c:85, cl-helper.h:47-55) and its secular
 * bracket search `while (gamma_max < 0)` has no bound
 * (Calculations-Parallel.c:208, 300).  Limits of a handle, in this order:
 *   [0] FP64 iterations per secular root in stage 2 (1..80, default 80);
 *       a root that has not converged by then gives DDCSVD_ERR_NOCONV
 *   [1] wall-clock limit of one device-side wait of the cooperative kernels
 *       (grid barriers) in microseconds (0..4000000; 0 = the built-in 4 s);
 *       a wait that runs out gives DDCSVD_ERR_TIMEOUT and the kernel returns
 *   [2] device workspace budget of the handle in bytes (0 = none); a call
 *       whose workspace would exceed it gives DDCSVD_ERR_ALLOC
 *   [3] fault injection for tests of the timeout path (0 in normal use):
 *       the first grid barrier of every cooperative launch waits for this
 *       many arrivals beyond its own CTAs, so its waits run out after limit
 *       [1] and the call returns DDCSVD_ERR_TIMEOUT
 * After any of these failures the handle stays usable.  get/set copy up to
 * `count` limits; set checks the ranges (DDCSVD_ERR_ARG, nothing changed). */
int ddcsvd_set_limits(ddcsvd_handle_t handle, const long long *values, int count);
int ddcsvd_get_limits(ddcsvd_handle_t handle, long long *values, int count);

/* ---------------------------------------------------------------- GEMM back ends */

/* The GEMM back ends of the pipeline, exposed for validation and reuse:
 * C (M x N, column-major, ldc) = beta*C + alpha * A B^T, with A (M x K) and
 * B (N x K) row-major (K contiguous; row r of A at A + r*lda), FP32 device
 * pointers.  mode: DDCSVD_MODE_BLOCKED_FP32 (CUDA cores), _BLOCKED_TF32X3 or
 * _BLOCKED_TF32X6 (tcgen05 tensor cores; lda, ldb multiples of 4 and 16-byte
 * aligned A, B). */
int ddcsvd_gemm_f32_device(ddcsvd_handle_t handle, int mode, int M, int N, int K, const float *A, int lda,
                           const float *B, int ldb, float *C, int ldc, float alpha, float beta);

/* ---------------------------------------------------------------- diagnostics */

const char *ddcsvd_status_string(int status);
/* Last error description on the calling thread ("" if none). */
const char *ddcsvd_last_error(void);
/* Number of kernels this library launched since load (for launch accounting). */
long long ddcsvd_kernel_launch_count(void);
/* Device time (ms) of the stages of the last ddcsvd_svd_f32_device call on the
 * handle when timing is enabled: [bidiag, sigma, vectors, back-transform]. */
int ddcsvd_set_stage_timing(ddcsvd_handle_t handle, int enable);
int ddcsvd_get_stage_times(ddcsvd_handle_t handle, float *ms4);
/* With timing enabled: summed device time (ms) and launch count per kernel
 * class of the last SVD on the handle: [0] bidiagonalisation kernels,
 * [1] trailing-update GEMMs, [2] D&C kernel, [3] vector kernels,
 * [4] back-transformation.  nclass <= 8. */
int ddcsvd_get_kernel_times(ddcsvd_handle_t handle, float *ms, int *launches, int nclass);

#ifdef __cplusplus
}
#endif

#endif /* DDCSVD_H */
