// api.cu -- handles, workspace, the five-stage pipeline and the C ABI.
//
// Pipeline (svd_gpu.c:99-121 order), m >= n (m < n runs on A^T):
//   1. bidiagonalisation (FP32)                      bidiag.cu
//   2. singular values by double D&C (FP64)          dc.cu
//   3-4. right/left vectors of B (FP64 core)         twisted.cu
//   5. back-transformation U = Q [Y;0], V = P X      backxform.cu
// All stages are enqueued on the handle's stream; the only host sync is the
// final read of the device status word.
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "internal.hpp"
#include "prep.hpp"

namespace ddcsvd {

long long g_launch_count = 0;
static thread_local std::string t_last_error;

void set_last_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_last_error = buf;
}

void ktimer_begin(ddcsvd_context* ctx, int cls) {
  if (!ctx->timing) return;
  if ((size_t)(2 * ctx->kused + 2) > ctx->kev.size()) {
    for (int k = 0; k < 64; k++) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return;
      ctx->kev.push_back(e);
    }
  }
  if ((int)ctx->kcat.size() <= ctx->kused) ctx->kcat.resize(ctx->kused + 1);
  ctx->kcat[ctx->kused] = cls;
  cudaEventRecord(ctx->kev[2 * ctx->kused], ctx->stream);
}

void ktimer_end(ddcsvd_context* ctx) {
  if (!ctx->timing || (size_t)(2 * ctx->kused + 2) > ctx->kev.size()) return;
  cudaEventRecord(ctx->kev[2 * ctx->kused + 1], ctx->stream);
  ctx->kused++;
}

void ktimer_collect(ddcsvd_context* ctx) {
  if (!ctx->timing) return;
  for (int c = 0; c < 8; c++) { ctx->kern_ms[c] = 0.f; ctx->kern_n[c] = 0; }
  for (int i = 0; i < ctx->kused; i++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->kev[2 * i], ctx->kev[2 * i + 1]) == cudaSuccess) {
      ctx->kern_ms[ctx->kcat[i]] += ms;
      ctx->kern_n[ctx->kcat[i]] += 1;
    }
  }
  ctx->kused = 0;
}

int ensure_workspace(ddcsvd_context* ctx, size_t bytes) {
  if (bytes <= ctx->ws_bytes) return DDCSVD_OK;
  if (ctx->ws_cap && bytes > ctx->ws_cap) {
    set_last_error("device workspace of %zu bytes exceeds the handle's workspace limit of %zu bytes", bytes,
                   ctx->ws_cap);
    return DDCSVD_ERR_ALLOC;
  }
  if (ctx->ws) {
    DDC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->ws);
    ctx->ws = nullptr;
    ctx->ws_bytes = 0;
  }
  size_t want = (size_t)round_up((long long)bytes, 1 << 21);
  if (ctx->ws_cap) want = std::min(want, ctx->ws_cap);
  if (cudaMalloc(&ctx->ws, want) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("device workspace of %zu bytes could not be allocated", want);
    return DDCSVD_ERR_ALLOC;
  }
  ctx->ws_bytes = want;
  return DDCSVD_OK;
}

int ensure_pinned(ddcsvd_context* ctx, size_t bytes) {
  if (bytes <= ctx->pinned_bytes) return DDCSVD_OK;
  if (ctx->pinned) {
    DDC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    cudaFreeHost(ctx->pinned);
    ctx->pinned = nullptr;
    ctx->pinned_bytes = 0;
  }
  size_t want = (size_t)round_up((long long)bytes, 1 << 20);
  if (cudaMallocHost(&ctx->pinned, want) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("pinned host buffer of %zu bytes could not be allocated", want);
    return DDCSVD_ERR_ALLOC;
  }
  ctx->pinned_bytes = want;
  return DDCSVD_OK;
}

// Clears the error code and writes the handle's limits (kernel arguments, so
// the host values may change right after the launch).
__global__ void status_init_kernel(DevStatus* st, unsigned wait_us, unsigned extra) {
  if (threadIdx.x == 0) *st = DevStatus{0, 0, wait_us, extra};
}

int reset_status(ddcsvd_context* ctx) {
  status_init_kernel<<<1, 32, 0, ctx->stream>>>(ctx->d_status, ctx->wait_us, ctx->barrier_extra);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

int check_status(ddcsvd_context* ctx, const char* stage) {
  DDC_CUDA_TRY(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost,
                               ctx->stream));
  DDC_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (ctx->h_status->code != 0) {
    set_last_error("%s: device status %d (detail %d)", stage, ctx->h_status->code, ctx->h_status->detail);
    return ctx->h_status->code;
  }
  return DDCSVD_OK;
}

static GemmKind kind_of(int mode) {
  switch (mode) {
    case DDCSVD_MODE_BLOCKED_TF32X3: return GEMM_TF32X3;
    case DDCSVD_MODE_BLOCKED_BF16X3: return GEMM_BF16X3;
    case DDCSVD_MODE_BLOCKED_TF32X6: return GEMM_TF32X6;
    default: return GEMM_SIMT;
  }
}

static int resolve_mode(int mode) {
  if (mode != DDCSVD_MODE_AUTO) return mode;
  const char* e = getenv("DDCSVD_MODE");
  if (e) {
    if (!strcmp(e, "plain")) return DDCSVD_MODE_PLAIN_FP32;
    if (!strcmp(e, "blocked")) return DDCSVD_MODE_BLOCKED_FP32;
    if (!strcmp(e, "tf32x3")) return DDCSVD_MODE_BLOCKED_TF32X3;
    if (!strcmp(e, "bf16x3")) return DDCSVD_MODE_BLOCKED_BF16X3;
    if (!strcmp(e, "tf32x6")) return DDCSVD_MODE_BLOCKED_TF32X6;
  }
  return DDCSVD_MODE_BLOCKED_TF32X6;
}

// ---------------------------------------------------------------- small kernels
// W = A with zero rows m .. ldw-1; with `st` set, a non-finite entry also
// records DDCSVD_ERR_NONFINITE (the input check rides on the copy's read).
__global__ void copy_pad_kernel(int m, int n, const float* __restrict__ A, int lda, float* W, int ldw,
                                DevStatus* st = nullptr) {
  const int c = blockIdx.y;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < ldw; r += gridDim.x * blockDim.x) {
    const float v = (r < m) ? A[r + (size_t)c * lda] : 0.f;
    if (st && !isfinite(v)) set_error(st, DDCSVD_ERR_NONFINITE, (int)((r + (size_t)c * m) % 2147483647));
    W[r + (size_t)c * ldw] = v;
  }
}

__global__ void sigma_out_kernel(int n, const double* s, float* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = (float)s[i];
}

__global__ void zero_rows_kernel(int r0, int r1, int ncols, float* C, int ldc) {
  const int c = blockIdx.y;
  for (int r = r0 + blockIdx.x * blockDim.x + threadIdx.x; r < r1; r += gridDim.x * blockDim.x)
    C[r + (size_t)c * ldc] = 0.f;
}

// R (n x n) = upper triangle of the first n rows of W
__global__ void triu_kernel(int n, const float* __restrict__ W, int ldw, float* R, int ldr) {
  const int c = blockIdx.y;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < ldr; r += gridDim.x * blockDim.x)
    R[r + (size_t)c * ldr] = (r <= c && r < n) ? W[r + (size_t)c * ldw] : 0.f;
}

// ---------------------------------------------------------------- pipeline
struct Plan {
  float *W, *d, *e, *tauq, *taup;
  double *sig_slot, *sig;
  char* blob;  // device copy of the bidiagonal preparation (prep.hpp)
  BidiagWork bw;
};

static int stage_event(ddcsvd_context* ctx, int k) {
  if (ctx->timing) DDC_CUDA_TRY(cudaEventRecord(ctx->ev[k], ctx->stream));
  return DDCSVD_OK;
}

// Full SVD of the m x n (m >= n) device matrix dA.  Workspace: region A
// (matrix, bidiagonal, sigma) persists through the call; region B is scratch
// reused by each stage in turn.
static int svd_core_impl(ddcsvd_context* ctx, int m, int n, const float* dA, int lda, float* dS, float* dU,
                         int ldu, float* dV, int ldv, int mode, bool check_finite);
static bool use_tall_qr(const ddcsvd_context* ctx, int m, int n, int mode);
static int svd_tall_qr(ddcsvd_context* ctx, int m, int n, const float* dA, int lda, float* dS, float* dU, int ldu,
                       float* dV, int ldv, int mode, bool check_finite);

__global__ void copy2d_kernel(int rows, int cols, const float* __restrict__ src, int lds, float* dst, int ldd) {
  const int c = blockIdx.y;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
    dst[r + (size_t)c * ldd] = src[r + (size_t)c * lds];
}

// The tensor-core back-transformation reads U and V through TMA, which needs
// 16-byte aligned bases and leading dimensions; other layouts go through
// aligned staging buffers.
static int svd_core(ddcsvd_context* ctx, int m, int n, const float* dA, int lda, float* dS, float* dU,
                    int ldu, float* dV, int ldv, int mode, bool check_finite) {
  const bool tcmode = (mode >= DDCSVD_MODE_BLOCKED_TF32X3);
  auto ok = [](const float* p, int ld) { return ((reinterpret_cast<uintptr_t>(p) & 15) == 0) && (ld % 4 == 0); };
  const bool tall = use_tall_qr(ctx, m, n, mode);
  if (!tcmode || (ok(dU, ldu) && ok(dV, ldv)))
    return tall ? svd_tall_qr(ctx, m, n, dA, lda, dS, dU, ldu, dV, ldv, mode, check_finite)
                : svd_core_impl(ctx, m, n, dA, lda, dS, dU, ldu, dV, ldv, mode, check_finite);
  const int lu = (int)round_up(m, 4), lv = (int)round_up(n, 4);
  float* buf = nullptr;
  DDC_CUDA_TRY(pool_alloc(ctx, &buf, sizeof(float) * ((size_t)lu * n + (size_t)lv * n + 64)));
  float* Ui = buf;
  float* Vi = buf + (size_t)lu * n + 32;
  auto v_copy = std::move(ctx->v_copy);  // the staged V is final only after the copy below
  ctx->v_copy = nullptr;
  int rc = tall ? svd_tall_qr(ctx, m, n, dA, lda, dS, Ui, lu, Vi, lv, mode, check_finite)
                : svd_core_impl(ctx, m, n, dA, lda, dS, Ui, lu, Vi, lv, mode, check_finite);
  ctx->v_copy = std::move(v_copy);
  if (rc == DDCSVD_OK) {
    copy2d_kernel<<<dim3(ceil_div(m, 256), n), 256, 0, ctx->stream>>>(m, n, Ui, lu, dU, ldu);
    copy2d_kernel<<<dim3(ceil_div(n, 256), n), 256, 0, ctx->stream>>>(n, n, Vi, lv, dV, ldv);
    count_launch(2);
  }
  cudaFreeAsync(buf, ctx->stream);
  if (rc == DDCSVD_OK) rc = check_status(ctx, "svd");
  return rc;
}

// Work forked onto the handle's side stream: fork() orders it after what the
// main stream has queued, the work is launched with the side stream standing
// in for the main one, and join() (at the latest when the object goes out of
// scope, error returns included) orders the main stream after it.
struct SideWork {
  ddcsvd_context* c;
  cudaStream_t main = nullptr;  // may be the legacy default stream (null)
  bool swapped = false, forked = false, joined = false;
  explicit SideWork(ddcsvd_context* ctx) : c(ctx) {}
  int fork() {
    DDC_CUDA_TRY(cudaEventRecord(c->fork_ev, c->stream));
    DDC_CUDA_TRY(cudaStreamWaitEvent(c->side, c->fork_ev, 0));
    forked = true;
    main = c->stream;
    c->stream = c->side;
    swapped = true;
    return DDCSVD_OK;
  }
  void back() {
    if (swapped) c->stream = main;
    swapped = false;
  }
  int join() {
    back();
    if (!forked || joined) return DDCSVD_OK;
    joined = true;
    DDC_CUDA_TRY(cudaEventRecord(c->join_ev, c->side));
    DDC_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->join_ev, 0));
    return DDCSVD_OK;
  }
  ~SideWork() { join(); }
};

static int svd_core_impl(ddcsvd_context* ctx, int m, int n, const float* dA, int lda, float* dS, float* dU,
                         int ldu, float* dV, int ldv, int mode, bool check_finite) {
  const bool plain = (mode == DDCSVD_MODE_PLAIN_FP32);
  const GemmKind kind = kind_of(mode);
  const int nctas = bidiag_coop_ctas(ctx, m, n);
  const int ldw = (int)round_up(m, 32);
  const size_t gsc = gemm_scratch_bytes(kind, m, n, 2 * kPanel);
  // Tensor-core modes prepare the back-transformation's WY blocks on the
  // side stream while stages 2-4 run (FP64-bound D&C, and a vector kernel
  // that leaves most of the GPU idle); their buffers then get a region of
  // their own instead of sharing the one that stages 2-4 use.  Stage timing
  // keeps everything on one stream so that the stage events mean what they say.
  const bool overlap = !plain && kind != GEMM_SIMT && !ctx->timing;
  BxPrepared bxl, bxr;
  auto region_a = [&](Arena& a, Plan& pl) {
    pl.W = a.take<float>((size_t)ldw * n);
    pl.d = a.take<float>(n + 4);
    pl.e = a.take<float>(n + 4);
    pl.tauq = a.take<float>(n + 4);
    pl.taup = a.take<float>(n + 4);
    pl.sig_slot = a.take<double>(n + 4);
    pl.sig = a.take<double>(n + 4);
    pl.blob = a.take<char>(prep_bounds({n}).blob_bytes);
    if (overlap) {
      bx_plan(m, n, n, kind, a, &bxl);
      bx_plan(n, std::max(0, n - 2), n, kind, a, &bxr);
    }
  };
  // ---- size
  Plan pl;
  size_t need;
  {
    Arena a;
    region_a(a, pl);
    Arena b1 = a;
    plan_bidiag(b1, m, n, ldw, nctas, kind, &pl.bw);
    b1.take<char>(gsc);
    Arena b2 = a;
    DDC_TRY(dc_sigma(ctx, n, nullptr, nullptr, nullptr, nullptr, nullptr, b2, true));
    Arena b3 = a;
    DDC_TRY(bd_vectors(ctx, n, (long long)n * n, nullptr, nullptr, nullptr, nullptr, nullptr, b3, true));
    Arena b4 = a, b5 = a;  // stage 5 (its buffers are in region a when it overlaps stages 2-4)
    if (!overlap) {
      DDC_TRY(apply_left_reflectors(ctx, m, n, nullptr, ldw, nullptr, dU, ldu, n, kind, plain, b4, true));
      DDC_TRY(apply_right_reflectors(ctx, n, std::max(0, n - 2), nullptr, ldw, nullptr, dV, ldv, n, kind, plain, b5,
                                     true));
    }
    need = std::max(std::max(b1.off, b2.off), std::max(std::max(b3.off, b4.off), b5.off));
  }
  DDC_TRY(ensure_workspace(ctx, need + 4096));
  Arena a;
  a.plan = false;
  a.base = (char*)ctx->ws;
  region_a(a, pl);
  // ---- stage 1
  if (!ctx->nested) {
    DDC_TRY(reset_status(ctx));
    ctx->kused = 0;
  }
  DDC_TRY(stage_event(ctx, 0));
  copy_pad_kernel<<<dim3(ceil_div(ldw, 256), n), 256, 0, ctx->stream>>>(m, n, dA, lda, pl.W, ldw,
                                                                      check_finite ? ctx->d_status : nullptr);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  {
    Arena b = a;
    plan_bidiag(b, m, n, ldw, nctas, kind, &pl.bw);
    Arena sc;
    sc.base = b.take<char>(gsc);
    sc.plan = false;
    sc.cap = gsc;
    if (plain) DDC_TRY(bidiag_plain(ctx, m, n, pl.W, ldw, pl.d, pl.e, pl.tauq, pl.taup, pl.bw));
    else DDC_TRY(bidiag_blocked(ctx, m, n, pl.W, ldw, pl.d, pl.e, pl.tauq, pl.taup, pl.bw, kind, &sc));
  }
  DDC_TRY(stage_event(ctx, 1));
  SideWork side(ctx);
  if (overlap) {
    DDC_TRY(side.fork());
    int rc = bx_prepare(ctx, 0, m, n, pl.W, ldw, pl.tauq, bxl);
    if (rc == DDCSVD_OK) rc = bx_prepare(ctx, 1, n, std::max(0, n - 2), pl.W, ldw, pl.taup, bxr);
    side.back();
    DDC_TRY(rc);
  }
  // ---- bidiagonal read-back: split at negligible superdiagonal entries and
  //      build the D&C forest and vector layout on the host (2n floats down, one blob up)
  const PrepBounds PB = prep_bounds({n});
  Prep P;
  {
    const size_t rb = (size_t)round_up(sizeof(float) * 2 * (n + 4), 256);
    const size_t ab = (size_t)round_up(sizeof(double) * 2 * (n + 4), 256);
    DDC_TRY(ensure_pinned(ctx, rb + ab + PB.blob_bytes));
    float* hd = (float*)ctx->pinned;
    float* he = hd + n + 4;
    DDC_CUDA_TRY(cudaMemcpyAsync(hd, pl.d, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (n > 1)
      DDC_CUDA_TRY(cudaMemcpyAsync(he, pl.e, sizeof(float) * (n - 1), cudaMemcpyDeviceToHost, ctx->stream));
    // the status word rides along: a stage-1 failure (non-finite input, a
    // wait that ran out) ends the call here instead of feeding stages 2-5
    DDC_TRY(check_status(ctx, "bidiagonalisation"));
    double* a64 = (double*)((char*)ctx->pinned + rb);
    double* b64 = a64 + n + 4;
    for (int i = 0; i < n; i++) {
      a64[i] = hd[i];
      b64[i] = (i < n - 1) ? (double)he[i] : 0.0;  // beta[N-1] := 0 (square case)
    }
    char* hb = (char*)ctx->pinned + rb + ab;
    DDC_TRY(prep_build(ctx, {n}, {GroupOut{dV, ldv, dU, ldu}}, a64, b64, FLT_EPSILON, false, hb, pl.blob, &P));
  }
  // ---- stage 2
  {
    Arena b = a;
    DDC_TRY(dc_sigma(ctx, n, P.b1, P.b2, pl.sig_slot, &P.H, P.dints, b, false));
  }
  DDC_TRY(stage_event(ctx, 2));
  // ---- stages 3-4: X straight into V, Y into the top of U (ascending order)
  {
    Arena b = a;
    DDC_TRY(bd_vectors(ctx, n, P.store, P.b1, P.b2, pl.sig_slot, &P.L, pl.sig, b, false));
  }
  if (m > n) {
    zero_rows_kernel<<<dim3(std::min(ceil_div(m - n, 256), 64), n), 256, 0, ctx->stream>>>(n, m, n, dU, ldu);
    count_launch();
  }
  DDC_TRY(stage_event(ctx, 3));
  // ---- stage 5: V first (its host copy may then overlap U's products)
  auto v_done = [&]() -> int {
    if (ctx->v_copy && !ctx->v_copy_started) {
      DDC_CUDA_TRY(cudaEventRecord(ctx->v_ready, ctx->stream));
      DDC_CUDA_TRY(cudaStreamWaitEvent(ctx->side, ctx->v_ready, 0));
      ctx->v_copy_started = true;
      DDC_CUDA_TRY(ctx->v_copy(ctx->side));
    }
    return DDCSVD_OK;
  };
  if (overlap) {
    DDC_TRY(side.join());
    ktimer_begin(ctx, KC_BACKXFORM);
    DDC_TRY(bx_apply(ctx, n, std::max(0, n - 2), bxr, dV, ldv, n, kind));
    DDC_TRY(v_done());
    DDC_TRY(bx_apply(ctx, m, n, bxl, dU, ldu, n, kind));
    ktimer_end(ctx);
  } else {
    Arena c = a;
    DDC_TRY(apply_right_reflectors(ctx, n, std::max(0, n - 2), pl.W, ldw, pl.taup, dV, ldv, n, kind, plain, c, false));
    DDC_TRY(v_done());
    Arena b = a;
    DDC_TRY(apply_left_reflectors(ctx, m, n, pl.W, ldw, pl.tauq, dU, ldu, n, kind, plain, b, false));
  }
  sigma_out_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(n, pl.sig, dS);
  count_launch();
  DDC_TRY(stage_event(ctx, 4));
  DDC_CUDA_TRY(cudaGetLastError());
  int rc = check_status(ctx, "svd");
  if (ctx->timing && rc == DDCSVD_OK) {
    for (int k = 0; k < 4; k++) cudaEventElapsedTime(&ctx->stage_ms[k], ctx->ev[k], ctx->ev[k + 1]);
    if (!ctx->nested) ktimer_collect(ctx);
  }
  return rc;
}

// Tall matrices (m >= 2n): Householder QR first (one-barrier-per-column panel
// kernel, tensor-core trailing updates), the SVD of the n x n factor R, then
// U = Q [U_R; 0] with the QR reflectors (the back-transformation machinery).
// The bidiagonalisation then runs on n x n instead of m x n: the GEMV half
// moves 2 * 4 * n^3 / 3 bytes instead of 2 * 4 * (m - n/3) n^2 / 2.
static bool use_tall_qr(const ddcsvd_context* ctx, int m, int n, int mode) {
  if (mode < DDCSVD_MODE_BLOCKED_TF32X3 || m < 2 * n || n < 128) return false;
  const int k = ctx->tune[TK_TALL_QR];
  // auto: when the matrix no longer fits the L2-resident regime of the
  // one-stage GEMVs (measured: 16384 x 8192 gains 1.3x, 8192 x 4096 loses 10%)
  return k == 1 || (k == 2 && (long long)m * n >= (64ll << 20));
}

static int svd_tall_qr(ddcsvd_context* ctx, int m, int n, const float* dA, int lda, float* dS, float* dU, int ldu,
                       float* dV, int ldv, int mode, bool check_finite) {
  const GemmKind kind = kind_of(mode);
  const int ldq = (int)round_up(m, 32), ldr = (int)round_up(n, 32);
  const int P = ctx->num_sms;
  Arena plan;
  plan.take<float>((size_t)ldq * n);      // Wq
  plan.take<float>(n + 4);                // tau
  plan.take<unsigned>(4);                 // amax
  plan.take<float>((size_t)ldr * n);      // R
  QrWork qw;
  plan_qr(plan, m, n, P, kind, &qw);
  char* buf = nullptr;
  if (pool_alloc(ctx, &buf, plan.off + 4096) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("device allocation of %zu bytes for the QR path failed", plan.off + 4096);
    return DDCSVD_ERR_ALLOC;
  }
  Arena a;
  a.plan = false;
  a.base = buf;
  float* Wq = a.take<float>((size_t)ldq * n);
  float* tau = a.take<float>(n + 4);
  unsigned* amax = a.take<unsigned>(4);
  float* R = a.take<float>((size_t)ldr * n);
  plan_qr(a, m, n, P, kind, &qw);
  int rc = DDCSVD_OK;
  do {
    if ((rc = reset_status(ctx))) break;
    ctx->kused = 0;
    copy_pad_kernel<<<dim3(ceil_div(ldq, 256), n), 256, 0, ctx->stream>>>(m, n, dA, lda, Wq, ldq,
                                                                          check_finite ? ctx->d_status : nullptr);
    count_launch();
    if ((rc = range_scale_matrix(ctx, m, n, Wq, ldq, amax))) break;
    if ((rc = qr_blocked(ctx, m, n, Wq, ldq, tau, qw, kind))) break;
    triu_kernel<<<dim3(ceil_div(ldr, 256), n), 256, 0, ctx->stream>>>(n, Wq, ldq, R, ldr);
    count_launch();
    ctx->nested = true;
    rc = svd_core_impl(ctx, n, n, R, ldr, dS, dU, ldu, dV, ldv, mode, false);
    ctx->nested = false;
    if (rc) break;
    // U = Q [U_R; 0]
    zero_rows_kernel<<<dim3(std::min(ceil_div(m - n, 256), 64), n), 256, 0, ctx->stream>>>(n, m, n, dU, ldu);
    count_launch();
    Arena p2;
    DDC_TRY(apply_left_reflectors(ctx, m, n, nullptr, ldq, nullptr, dU, ldu, n, kind, false, p2, true));
    if ((rc = ensure_workspace(ctx, p2.off + 4096))) break;
    Arena w2;
    w2.plan = false;
    w2.base = (char*)ctx->ws;
    if ((rc = apply_left_reflectors(ctx, m, n, Wq, ldq, tau, dU, ldu, n, kind, false, w2, false))) break;
    if ((rc = range_unscale_vector(ctx, n, dS, amax))) break;
    rc = check_status(ctx, "svd (QR path)");
  } while (0);
  ctx->nested = false;
  cudaFreeAsync(buf, ctx->stream);
  if (rc == DDCSVD_OK && ctx->timing) ktimer_collect(ctx);
  return rc;
}

__global__ void transpose_f32_kernel(int rows, int cols, const float* __restrict__ A, int lda, float* AT, int ldat) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int r = r0 + threadIdx.x, c = c0 + k;
    tile[k][threadIdx.x] = (r < rows && c < cols) ? A[r + (size_t)c * lda] : 0.f;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int c = c0 + threadIdx.x, r = r0 + k;
    if (r < rows && c < cols) AT[c + (size_t)r * ldat] = tile[threadIdx.x][k];
  }
}

static int svd_device(ddcsvd_context* ctx, int m, int n, const float* dA, int lda, float* dS, float* dU,
                      int ldu, float* dV, int ldv, int mode, float* dAT_scratch) {
  mode = resolve_mode(mode);
  if (mode < DDCSVD_MODE_PLAIN_FP32 || mode > DDCSVD_MODE_BLOCKED_TF32X6) return DDCSVD_ERR_ARG;
  if (mode >= DDCSVD_MODE_BLOCKED_TF32X3 && !tc_available(ctx)) {
    set_last_error("tensor-core mode requested but tcgen05 kernels are unavailable on this device");
    return DDCSVD_ERR_UNSUPPORTED;
  }
  if (m >= n) return svd_core(ctx, m, n, dA, lda, dS, dU, ldu, dV, ldv, mode, true);
  // m < n: SVD of A^T (n x m); U_A = V_{A^T}, V_A = U_{A^T}
  transpose_f32_kernel<<<dim3(ceil_div(m, 32), ceil_div(n, 32)), dim3(32, 8), 0, ctx->stream>>>(m, n, dA, lda,
                                                                                               dAT_scratch, n);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  return svd_core(ctx, n, m, dAT_scratch, n, dS, dV, ldv, dU, ldu, mode, true);
}

}  // namespace ddcsvd

using namespace ddcsvd;

// ---------------------------------------------------------------- handles
static std::mutex g_default_mu;
static ddcsvd_context* g_default[64] = {nullptr};

static int create_ctx(ddcsvd_context** out, int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device");
    return DDCSVD_ERR_NODEVICE;
  }
  if (device < 0) DDC_CUDA_TRY(cudaGetDevice(&device));
  if (device >= ndev) return DDCSVD_ERR_ARG;
  DDC_CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop;
  DDC_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) {
    set_last_error("device %d is sm_%d%d; this library is built for sm_103a", device, prop.major, prop.minor);
    return DDCSVD_ERR_NODEVICE;
  }
  ddcsvd_context* c = new ddcsvd_context();
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  c->smem_optin = prop.sharedMemPerBlockOptin;
  DDC_CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->own_stream = true;
  DDC_CUDA_TRY(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
  DDC_CUDA_TRY(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
  DDC_CUDA_TRY(cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming));
  DDC_CUDA_TRY(cudaEventCreateWithFlags(&c->v_ready, cudaEventDisableTiming));
  {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    DDC_CUDA_TRY(cudaMemPoolCreate(&c->pool, &props));
    unsigned long long keep = ~0ull;
    DDC_CUDA_TRY(cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  }
  DDC_CUDA_TRY(cudaMalloc(&c->d_status, sizeof(DevStatus)));
  DDC_CUDA_TRY(cudaMallocHost(&c->h_status, sizeof(DevStatus)));
  for (int k = 0; k < 5; k++) DDC_CUDA_TRY(cudaEventCreate(&c->ev[k]));
  *out = c;
  return DDCSVD_OK;
}

static int default_ctx(ddcsvd_context** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    set_last_error("no CUDA device");
    return DDCSVD_ERR_NODEVICE;
  }
  std::lock_guard<std::mutex> g(g_default_mu);
  if (dev < 0 || dev >= 64) return DDCSVD_ERR_ARG;
  if (!g_default[dev]) DDC_TRY(create_ctx(&g_default[dev], dev));
  *out = g_default[dev];
  return DDCSVD_OK;
}

extern "C" {

const char* ddcsvd_status_string(int s) {
  switch (s) {
    case DDCSVD_OK: return "ok";
    case DDCSVD_ERR_ARG: return "invalid argument";
    case DDCSVD_ERR_CUDA: return "CUDA error";
    case DDCSVD_ERR_ALLOC: return "allocation failed";
    case DDCSVD_ERR_NOCONV: return "iteration did not converge";
    case DDCSVD_ERR_TIMEOUT: return "device wait timed out";
    case DDCSVD_ERR_NODEVICE: return "no usable device";
    case DDCSVD_ERR_NONFINITE: return "input holds NaN or Inf";
    case DDCSVD_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char* ddcsvd_last_error(void) { return t_last_error.c_str(); }

long long ddcsvd_kernel_launch_count(void) { return __atomic_load_n(&g_launch_count, __ATOMIC_RELAXED); }

int ddcsvd_create(ddcsvd_handle_t* handle, int device) {
  if (!handle) return DDCSVD_ERR_ARG;
  return create_ctx(handle, device);
}

int ddcsvd_destroy(ddcsvd_handle_t h) {
  if (!h) return DDCSVD_ERR_ARG;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  if (h->ws) cudaFree(h->ws);
  if (h->pinned) cudaFreeHost(h->pinned);
  if (h->d_status) cudaFree(h->d_status);
  if (h->h_status) cudaFreeHost(h->h_status);
  for (int k = 0; k < 5; k++) if (h->ev[k]) cudaEventDestroy(h->ev[k]);
  if (h->side) {
    cudaStreamSynchronize(h->side);
    cudaStreamDestroy(h->side);
  }
  if (h->fork_ev) cudaEventDestroy(h->fork_ev);
  if (h->join_ev) cudaEventDestroy(h->join_ev);
  if (h->v_ready) cudaEventDestroy(h->v_ready);
  if (h->own_stream) cudaStreamDestroy(h->stream);
  if (h->pool) cudaMemPoolDestroy(h->pool);
  delete h;
  return DDCSVD_OK;
}

int ddcsvd_set_stream(ddcsvd_handle_t h, void* stream) {
  if (!h) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  if (h->own_stream) {
    cudaStreamSynchronize(h->stream);
    cudaStreamDestroy(h->stream);
    h->own_stream = false;
  }
  // NULL selects the legacy default stream (what torch calls stream 0)
  h->stream = (cudaStream_t)stream;
  return DDCSVD_OK;
}

int ddcsvd_release_workspace(ddcsvd_handle_t h) {
  if (!h) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  cudaStreamSynchronize(h->stream);
  if (h->ws) cudaFree(h->ws);
  h->ws = nullptr;
  h->ws_bytes = 0;
  if (h->pool) cudaMemPoolTrimTo(h->pool, 0);
  return DDCSVD_OK;
}

int ddcsvd_set_limits(ddcsvd_handle_t h, const long long* values, int count) {
  if (!h || !values || count < 0) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  t_last_error.clear();
  long long v[4] = {h->sec_maxit, (long long)h->wait_us, (long long)h->ws_cap, (long long)h->barrier_extra};
  for (int k = 0; k < std::min(count, 4); k++) v[k] = values[k];
  if (v[0] < 1 || v[0] > 80 || v[1] < 0 || v[1] > 4000000 || v[2] < 0 || v[3] < 0 || v[3] > 1024) {
    set_last_error("limits out of range: iterations 1..80, wait 0..4000000 us, workspace >= 0, arrivals 0..1024");
    return DDCSVD_ERR_ARG;
  }
  h->sec_maxit = (int)v[0];
  h->wait_us = (unsigned)v[1];
  h->ws_cap = (size_t)v[2];
  h->barrier_extra = (unsigned)v[3];
  return DDCSVD_OK;
}

int ddcsvd_get_limits(ddcsvd_handle_t h, long long* values, int count) {
  if (!h || !values || count < 0) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  const long long v[4] = {h->sec_maxit, (long long)h->wait_us, (long long)h->ws_cap, (long long)h->barrier_extra};
  for (int k = 0; k < std::min(count, 4); k++) values[k] = v[k];
  return DDCSVD_OK;
}

int ddcsvd_set_stage_timing(ddcsvd_handle_t h, int enable) {
  if (!h) return DDCSVD_ERR_ARG;
  h->timing = enable != 0;
  return DDCSVD_OK;
}

int ddcsvd_get_kernel_times(ddcsvd_handle_t h, float* ms, int* launches, int nclass) {
  if (!h || !ms || nclass < 0) return DDCSVD_ERR_ARG;
  for (int c = 0; c < nclass && c < 8; c++) {
    ms[c] = h->kern_ms[c];
    if (launches) launches[c] = h->kern_n[c];
  }
  return DDCSVD_OK;
}

int ddcsvd_get_stage_times(ddcsvd_handle_t h, float* ms4) {
  if (!h || !ms4) return DDCSVD_ERR_ARG;
  for (int k = 0; k < 4; k++) ms4[k] = h->stage_ms[k];
  return DDCSVD_OK;
}

int ddcsvd_svd_f32_device(ddcsvd_handle_t h, int m, int n, const float* dA, int lda, float* dSigma,
                          float* dU, int ldu, float* dV, int ldv, int mode) {
  t_last_error.clear();
  if (!h || m <= 0 || n <= 0 || !dA || !dSigma || !dU || !dV) return DDCSVD_ERR_ARG;
  if (lda < m || ldu < m || ldv < n) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  float* at = nullptr;
  if (m < n) {
    // A^T scratch lives in its own allocation so the pipeline workspace stays intact
    DDC_CUDA_TRY(pool_alloc(h, &at, sizeof(float) * (size_t)m * n));
  }
  int rc = svd_device(h, m, n, dA, lda, dSigma, dU, ldu, dV, ldv, mode, at);
  if (at) cudaFreeAsync(at, h->stream);
  return rc;
}

static int bidiag_device(ddcsvd_context* h, int m, int n, float* dA, int lda, float* dD, float* dE,
                         float* dTauq, float* dTaup, int mode) {
  mode = resolve_mode(mode);
  if (mode >= DDCSVD_MODE_BLOCKED_TF32X3 && !tc_available(h)) return DDCSVD_ERR_UNSUPPORTED;
  const GemmKind kind = kind_of(mode);
  BidiagWork bw;
  size_t scb = gemm_scratch_bytes(kind, m, n, 2 * kPanel);
  char* sc = nullptr;
  for (int pass = 0; pass < 2; pass++) {
    Arena a;
    a.plan = pass == 0;
    a.base = (char*)h->ws;
    plan_bidiag(a, m, n, lda, bidiag_coop_ctas(h, m, n), kind, &bw);
    sc = a.take<char>(scb);
    if (pass == 0) DDC_TRY(ensure_workspace(h, a.off + 4096));
  }
  DDC_TRY(reset_status(h));
  Arena s;
  s.base = sc;
  s.plan = false;
  s.cap = scb;
  if (mode == DDCSVD_MODE_PLAIN_FP32) DDC_TRY(bidiag_plain(h, m, n, dA, lda, dD, dE, dTauq, dTaup, bw));
  else DDC_TRY(bidiag_blocked(h, m, n, dA, lda, dD, dE, dTauq, dTaup, bw, kind, &s));
  return check_status(h, "bidiag");
}

int ddcsvd_bidiag_f32_device(ddcsvd_handle_t h, int m, int n, float* dA, int lda, float* dD, float* dE,
                             float* dTauq, float* dTaup, int mode) {
  if (!h || m <= 0 || n <= 0 || m < n || lda < m || (lda % 4) != 0) return DDCSVD_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(dA) & 15) != 0) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  return bidiag_device(h, m, n, dA, lda, dD, dE, dTauq, dTaup, mode);
}

// Standalone stages 2-4 on a device FP64 bidiagonal: read it back, split it
// (FP64 tolerance), build the forest, run D&C (and the vectors if asked).
static int bd_standalone(ddcsvd_context* h, int N, const double* dB1, const double* dB2, bool square,
                         const double* dSigmaIn, double* dSigmaOut, float* dX, float* dY) {
  const PrepBounds PB = prep_bounds({N});
  size_t need;
  {
    Arena a;
    a.take<char>(PB.blob_bytes);
    a.take<double>(N + 4);
    Arena b = a, c = a;
    DDC_TRY(dc_sigma(h, N, nullptr, nullptr, nullptr, nullptr, nullptr, b, true));
    if (dX) DDC_TRY(bd_vectors(h, N, (long long)N * N, nullptr, nullptr, nullptr, nullptr, nullptr, c, true));
    c.take<int>(N + 8);
    need = std::max(b.off, c.off);
  }
  DDC_TRY(ensure_workspace(h, need + 4096));
  Arena a;
  a.plan = false;
  a.base = (char*)h->ws;
  char* blob = a.take<char>(PB.blob_bytes);
  double* sig_slot = a.take<double>(N + 4);
  const size_t ab = (size_t)round_up(sizeof(double) * 2 * (N + 4), 256);
  DDC_TRY(ensure_pinned(h, ab + PB.blob_bytes));
  double* a64 = (double*)h->pinned;
  double* b64 = a64 + N + 4;
  DDC_CUDA_TRY(cudaMemcpyAsync(a64, dB1, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
  DDC_CUDA_TRY(cudaMemcpyAsync(b64, dB2, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
  DDC_CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (square) b64[N - 1] = 0.0;
  Prep P;
  DDC_TRY(prep_build(h, {N}, {GroupOut{dX, N, dY, N}}, a64, b64, DBL_EPSILON, !square, (char*)h->pinned + ab, blob,
                     &P));
  DDC_TRY(reset_status(h));
  if (dX && P.single_block && dSigmaIn) {
    // one unreduced block: the caller's ascending sigma is already in slot order
    DDC_CUDA_TRY(cudaMemcpyAsync(sig_slot, dSigmaIn, sizeof(double) * N, cudaMemcpyDeviceToDevice, h->stream));
  } else {
    Arena b = a;
    DDC_TRY(dc_sigma(h, N, P.b1, P.b2, sig_slot, &P.H, P.dints, b, false));
  }
  if (dX) {
    Arena c = a;
    DDC_TRY(bd_vectors(h, N, P.store, P.b1, P.b2, sig_slot, &P.L, dSigmaOut, c, false));
  } else {
    Arena c = a;
    DDC_TRY(sort_values(h, N, sig_slot, dSigmaOut, &P.L, c));
  }
  return check_status(h, dX ? "bdvec" : "bdsdc");
}

// ---- host-only planning of stage 2 (no device work): what the pipeline does
// between the bidiagonal read-back and the D&C launch, for tests and tools
int ddcsvd_split_plan(int N, double* a, double* b, double eps, int* starts, int* nstarts) {
  t_last_error.clear();
  if (N <= 0 || !a || !b || !starts || !nstarts || !(eps >= 0.0)) return DDCSVD_ERR_ARG;
  std::vector<int> st, lo(N), hi(N);
  split_bidiagonal(N, a, b, eps, st, lo.data(), hi.data());
  for (size_t i = 0; i < st.size(); i++) starts[i] = st[i];
  *nstarts = (int)st.size();
  return DDCSVD_OK;
}

int ddcsvd_dc_plan(int N, int nstarts, const int* starts, int terms_per_lane, int* out, long long cap, int* meta) {
  t_last_error.clear();
  if (N <= 0 || nstarts < 2 || !starts || !meta || cap < 0 || (cap > 0 && !out)) return DDCSVD_ERR_ARG;
  if (starts[0] != 0 || starts[nstarts - 1] != N) return DDCSVD_ERR_ARG;
  for (int i = 0; i + 1 < nstarts; i++)
    if (starts[i + 1] < starts[i]) return DDCSVD_ERR_ARG;
  DcHost H;
  dc_build_host(N, std::vector<int>(starts, starts + nstarts), H, terms_per_lane);
  meta[0] = H.nnodes;
  meta[1] = H.maxdepth;
  meta[2] = H.ndm;
  meta[3] = H.ntrees;
  meta[4] = H.nseg;
  meta[5] = H.maxtree;
  meta[6] = (int)H.tree_off;
  meta[7] = (int)H.ints.size();
  if ((long long)H.ints.size() > cap) {
    set_last_error("node table needs %zu ints", H.ints.size());
    return DDCSVD_ERR_ARG;
  }
  for (size_t i = 0; i < H.ints.size(); i++) out[i] = H.ints[i];
  return DDCSVD_OK;
}

int ddcsvd_bdsdc_sigma_device(ddcsvd_handle_t h, int N, const double* dB1, const double* dB2, double* dSigma) {
  if (!h || N <= 0 || !dB1 || !dB2 || !dSigma) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  return bd_standalone(h, N, dB1, dB2, false, nullptr, dSigma, nullptr, nullptr);
}

int ddcsvd_bdvec_device(ddcsvd_handle_t h, int N, const double* dA, const double* dB, const double* dSigma,
                        float* dX, float* dY) {
  if (!h || N <= 0 || !dA || !dB || !dSigma || !dX || !dY) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  double* scratch_sorted = nullptr;
  DDC_CUDA_TRY(pool_alloc(h, &scratch_sorted, sizeof(double) * N));
  int rc = bd_standalone(h, N, dA, dB, true, dSigma, scratch_sorted, dX, dY);
  cudaFreeAsync(scratch_sorted, h->stream);
  return rc;
}

int ddcsvd_gemm_f32_device(ddcsvd_handle_t h, int mode, int M, int N, int K, const float* A, int lda,
                           const float* B, int ldb, float* C, int ldc, float alpha, float beta) {
  if (!h || M < 0 || N < 0 || K < 0 || !A || !B || !C || lda < K || ldb < K || ldc < M) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  t_last_error.clear();
  if (mode != DDCSVD_MODE_BLOCKED_FP32 && mode != DDCSVD_MODE_BLOCKED_TF32X3 && mode != DDCSVD_MODE_BLOCKED_TF32X6)
    return DDCSVD_ERR_ARG;
  if (mode != DDCSVD_MODE_BLOCKED_FP32 && !tc_available(h)) return DDCSVD_ERR_UNSUPPORTED;
  const GemmKind kind = kind_of(mode);
  const size_t sb = gemm_scratch_bytes(kind, M, N, K);
  DDC_TRY(ensure_workspace(h, sb + 4096));
  Arena sc;
  sc.base = (char*)h->ws;
  sc.plan = false;
  sc.cap = sb;
  DDC_TRY(reset_status(h));
  Mat none{nullptr, 0, 0};
  if (kind == GEMM_SIMT) {
    DDC_TRY(gemm(h, kind, M, N, K, Mat{A, lda, 1}, Mat{B, 1, ldb}, 0, none, none, alpha, beta, C, ldc, &sc));
  } else {
    DDC_TRY(gemm_tc_kmajor(h, kind, M, N, K, A, lda, 0, B, ldb, 0, C, ldc, alpha, beta, &sc));
  }
  return check_status(h, "gemm");
}

// ---------------------------------------------------------------- host-buffer API
static int svd_host_f32(ddcsvd_context* h, int m, int n, const float* A, int lda, float* S, float* U, int ldu,
                        float* V, int ldv, int mode) {
  const int k = std::min(m, n);
  // device copies with 16-byte aligned bases and leading dimensions (the
  // tensor-core back-transformation then writes U and V in place)
  const int lum = (int)round_up(m, 4), lvn = (int)round_up(n, 4);
  const size_t na = (size_t)m * n, ns = round_up(k, 4), nu = (size_t)lum * k, nv = (size_t)lvn * k;
  float *dA = nullptr, *dS = nullptr, *dU = nullptr, *dV = nullptr;
  DDC_CUDA_TRY(pool_alloc(h, &dA, sizeof(float) * (round_up(na, 4) + ns + nu + nv + 64)));
  dS = dA + round_up(na, 4);
  dU = dS + ns;
  dV = dU + nu;
  // host copy of a device matrix (rows x k, device ld ldd) on stream st
  auto out2d = [&](float* dst, int ld, const float* src, int ldd, int rows, cudaStream_t st) {
    return (ld == rows && ldd == rows)
               ? cudaMemcpyAsync(dst, src, sizeof(float) * (size_t)rows * k, cudaMemcpyDeviceToHost, st)
               : cudaMemcpy2DAsync(dst, sizeof(float) * ld, src, sizeof(float) * ldd, sizeof(float) * rows, k,
                                   cudaMemcpyDeviceToHost, st);
  };
  int rc = DDCSVD_OK;
  bool side_used = false;
  do {
    if (lda == m) {
      if (cudaMemcpyAsync(dA, A, sizeof(float) * na, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
    } else {
      if (cudaMemcpy2DAsync(dA, sizeof(float) * m, A, sizeof(float) * lda, sizeof(float) * m, n,
                            cudaMemcpyHostToDevice, h->stream) != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
    }
    float* at = nullptr;
    if (m < n && pool_alloc(h, &at, sizeof(float) * na) != cudaSuccess) { rc = DDCSVD_ERR_ALLOC; break; }
    // the pipeline finishes its second output first (V, or U of a wide
    // input): the pipeline queues that copy on the side stream as soon as
    // the output is final (before the other output's products)
    const bool early_v = (m >= n);
    h->v_copy = [&](cudaStream_t st) {
      return early_v ? out2d(V, ldv, dV, lvn, n, st) : out2d(U, ldu, dU, lum, m, st);
    };
    h->v_copy_started = false;
    rc = svd_device(h, m, n, dA, m, dS, dU, lum, dV, lvn, mode, at);
    h->v_copy = nullptr;
    side_used = h->v_copy_started;
    if (at) cudaFreeAsync(at, h->stream);
    if (rc != DDCSVD_OK) break;
    if (!side_used) {
      const cudaError_t e = early_v ? out2d(V, ldv, dV, lvn, n, h->stream) : out2d(U, ldu, dU, lum, m, h->stream);
      if (e != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
    }
    if (cudaMemcpyAsync(S, dS, sizeof(float) * k, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
    {
      const cudaError_t e = early_v ? out2d(U, ldu, dU, lum, m, h->stream) : out2d(V, ldv, dV, lvn, n, h->stream);
      if (e != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
    }
  } while (0);
  if (side_used) {  // the side stream's copy ends before the buffers are released
    cudaEventRecord(h->join_ev, h->side);
    cudaStreamWaitEvent(h->stream, h->join_ev, 0);
  }
  if (rc == DDCSVD_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = DDCSVD_ERR_CUDA;
  cudaFreeAsync(dA, h->stream);
  cudaStreamSynchronize(h->stream);
  if (rc == DDCSVD_ERR_CUDA && t_last_error.empty()) set_last_error("CUDA copy failed");
  return rc;
}

int ddcsvd_svd_f32(int m, int n, const float* A, int lda, float* sigma, float* U, int ldu, float* V, int ldv,
                   int mode) {
  t_last_error.clear();
  if (m <= 0 || n <= 0 || !A || !sigma || !U || !V || lda < m || ldu < m || ldv < n) return DDCSVD_ERR_ARG;
  ddcsvd_context* h;
  DDC_TRY(default_ctx(&h));
  std::lock_guard<std::mutex> g(h->mu);
  return svd_host_f32(h, m, n, A, lda, sigma, U, ldu, V, ldv, mode);
}

int ddcsvd_svd_f32_host(ddcsvd_handle_t h, int m, int n, const float* A, int lda, float* sigma, float* U, int ldu,
                        float* V, int ldv, int mode) {
  t_last_error.clear();
  if (!h || m <= 0 || n <= 0 || !A || !sigma || !U || !V || lda < m || ldu < m || ldv < n) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  return svd_host_f32(h, m, n, A, lda, sigma, U, ldu, V, ldv, mode);
}

int svd_gpu_ex(int m, int n, double* A, double* sigma, double* U, double* V, int mode) {
  t_last_error.clear();
  if (m <= 0 || n <= 0 || !A || !sigma || !U || !V) return DDCSVD_ERR_ARG;
  ddcsvd_context* h;
  DDC_TRY(default_ctx(&h));
  std::lock_guard<std::mutex> g(h->mu);
  const int k = std::min(m, n);
  const size_t na = (size_t)m * n, nu = (size_t)m * k, nv = (size_t)n * k;
  // at least what the bidiagonal read-back inside the call asks for, so the
  // buffer is never reallocated under pa / pu / pv
  const size_t own = sizeof(float) * (na + k + nu + nv + 64);
  const size_t readback = (size_t)round_up(sizeof(float) * 2 * (k + 4), 256) +
                          (size_t)round_up(sizeof(double) * 2 * (k + 4), 256) + prep_bounds({k}).blob_bytes;
  DDC_TRY(ensure_pinned(h, std::max(own, readback)));
  float* pa = (float*)h->pinned;
  float* ps = pa + na;
  float* pu = ps + k;
  float* pv = pu + nu;
  for (size_t i = 0; i < na; i++) pa[i] = (float)A[i];
  int rc = svd_host_f32(h, m, n, pa, m, ps, pu, m, pv, n, mode);
  if (rc != DDCSVD_OK) return rc;
  for (int i = 0; i < k; i++) sigma[i] = ps[i];
  for (size_t i = 0; i < nu; i++) U[i] = pu[i];
  for (size_t i = 0; i < nv; i++) V[i] = pv[i];
  return DDCSVD_OK;
}

void svd_gpu(int m, int n, double* A, double* sigma, double* U, double* V) {
  int rc = svd_gpu_ex(m, n, A, sigma, U, V, DDCSVD_MODE_AUTO);
  if (rc != DDCSVD_OK) {
    fprintf(stderr, "svd_gpu: %s (%s)\n", ddcsvd_status_string(rc), ddcsvd_last_error());
    if (sigma && m > 0 && n > 0)
      for (int i = 0; i < std::min(m, n); i++) sigma[i] = __builtin_nan("");
  }
}

// Wide inputs (m < n, bidiag.c:130-155 / bidiag_par.c:361-383): the upper
// reduction of A to an m x (m+1) bidiagonal is the reduction of the tall
// C = [0 | A^T] (n x (m+1)) step for step.  Left reflector i of A is right
// reflector i of C (row i, columns i+1..m); right reflector i of A is left
// reflector i+1 of C; C's zero first column takes the identity; A's final
// "no reflection on the left" is C's "one element left, no reflection on
// the right" (bidiag.c:125-129); A's last right reflector is C's last left
// one.  So alpha_i = e_C[i], beta_i = d_C[i+1], A[i, j] = C[j, i+1].
void bidiag_par(int m, int n, double* A, double* alpha, double* beta) {
  t_last_error.clear();
  int rc = DDCSVD_OK;
  ddcsvd_context* h = nullptr;
  if (m <= 0 || n <= 0 || !A || !alpha || !beta) rc = DDCSVD_ERR_ARG;
  if (rc == DDCSVD_OK) rc = default_ctx(&h);
  if (rc == DDCSVD_OK) {
    std::lock_guard<std::mutex> g(h->mu);
    const bool wide = m < n;
    const int mc = wide ? n : m, nc = wide ? m + 1 : n;  // the tall matrix reduced on the GPU
    const int ldw = (int)round_up(mc, 32);
    const size_t na = (size_t)mc * nc;
    float* dW = nullptr;
    double* dOut = nullptr;
    do {
      if (pool_alloc(h, &dW, sizeof(float) * ((size_t)ldw * nc + 4 * (size_t)nc + 64)) != cudaSuccess) { rc = DDCSVD_ERR_ALLOC; break; }
      if (pool_alloc(h, &dOut, sizeof(double) * na) != cudaSuccess) { rc = DDCSVD_ERR_ALLOC; break; }
      float* dd = dW + (size_t)ldw * nc;
      float* de = dd + nc;
      float* tq = de + nc;
      float* tp = tq + nc;
      // [float copy of the input | 256-byte aligned FP64 reflectors]; d, e reuse the front
      rc = ensure_pinned(h, round_up(sizeof(float) * na, 256) + sizeof(double) * na + 64);
      if (rc) break;
      float* pa = (float*)h->pinned;
      if (!wide) {
        for (size_t i = 0; i < na; i++) pa[i] = (float)A[i];
      } else {
        for (int r = 0; r < mc; r++) pa[r] = 0.f;
        for (int c = 0; c < m; c++)
          for (int r = 0; r < n; r++) pa[r + (size_t)(c + 1) * mc] = (float)A[c + (size_t)r * m];
      }
      if (cudaMemsetAsync(dW, 0, sizeof(float) * (size_t)ldw * nc, h->stream) != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
      if (cudaMemcpy2DAsync(dW, sizeof(float) * ldw, pa, sizeof(float) * mc, sizeof(float) * mc, nc,
                            cudaMemcpyHostToDevice, h->stream) != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
      rc = bidiag_device(h, mc, nc, dW, ldw, dd, de, tq, tp, DDCSVD_MODE_AUTO);
      if (rc) break;
      rc = export_reflectors(h, mc, nc, dW, ldw, dd, de, tq, tp, dOut);
      if (rc) break;
      double* po = (double*)((char*)h->pinned + round_up(sizeof(float) * na, 256));
      float* pd = (float*)h->pinned;
      if (cudaMemcpyAsync(po, dOut, sizeof(double) * na, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
      if (cudaMemcpyAsync(pd, dd, sizeof(float) * 2 * nc, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
      if (cudaStreamSynchronize(h->stream) != cudaSuccess) { rc = DDCSVD_ERR_CUDA; break; }
      if (!wide) {
        memcpy(A, po, sizeof(double) * na);
        for (int i = 0; i < n; i++) alpha[i] = pd[i];
        for (int i = 0; i < n - 1; i++) beta[i] = pd[n + i];
      } else {
        for (int c = 0; c < m; c++)
          for (int r = 0; r < n; r++) A[c + (size_t)r * m] = po[r + (size_t)(c + 1) * mc];
        for (int i = 0; i < m; i++) {
          alpha[i] = pd[nc + i];
          beta[i] = pd[i + 1];
        }
      }
    } while (0);
    if (dW) cudaFreeAsync(dW, h->stream);
    if (dOut) cudaFreeAsync(dOut, h->stream);
    cudaStreamSynchronize(h->stream);
  }
  if (rc != DDCSVD_OK) {
    fprintf(stderr, "bidiag_par: %s (%s)\n", ddcsvd_status_string(rc), ddcsvd_last_error());
    for (int i = 0; m > 0 && n > 0 && i < std::min(m, n); i++) alpha[i] = __builtin_nan("");
  }
}

// form_u_par / form_v_par: the explicit factors from bidiag_par's reflectors
// (host FP64 buffers in and out, computed on the GPU in FP64).
static int form_factor_host(int m, int n, const double* A_mod, double* Q, bool left) {
  if (m <= 0 || n <= 0 || !A_mod || !Q) return DDCSVD_ERR_ARG;
  ddcsvd_context* h = nullptr;
  DDC_TRY(default_ctx(&h));
  std::lock_guard<std::mutex> g(h->mu);
  const int rows = left ? m : n;
  const size_t na = (size_t)m * n, nq = (size_t)rows * rows, ns = left ? 0 : (size_t)n * n;
  double* buf = nullptr;
  int rc = DDCSVD_OK;
  if (pool_alloc(h, &buf, sizeof(double) * (na + nq + ns + 16)) != cudaSuccess) {
    set_last_error("device allocation of %zu bytes failed", sizeof(double) * (na + nq + ns + 16));
    return DDCSVD_ERR_ALLOC;
  }
  double* dA = buf;
  double* dQ = buf + na;
  double* dS = dQ + nq;
  do {
    if (cudaMemcpyAsync(dA, A_mod, sizeof(double) * na, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) {
      rc = DDCSVD_ERR_CUDA;
      break;
    }
    rc = form_factor_f64(h, m, n, dA, left, dQ, dS);
    if (rc) break;
    if (cudaMemcpyAsync(Q, dQ, sizeof(double) * nq, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) {
      rc = DDCSVD_ERR_CUDA;
      break;
    }
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) rc = DDCSVD_ERR_CUDA;
  } while (0);
  cudaFreeAsync(buf, h->stream);
  cudaStreamSynchronize(h->stream);
  return rc;
}

void form_u_par(int m, int n, const double* A_mod, double* U) {
  t_last_error.clear();
  const int rc = form_factor_host(m, n, A_mod, U, true);
  if (rc != DDCSVD_OK) {
    fprintf(stderr, "form_u_par: %s (%s)\n", ddcsvd_status_string(rc), ddcsvd_last_error());
    if (U && m > 0) U[0] = __builtin_nan("");
  }
}

void form_v_par(int m, int n, const double* A_mod, double* V) {
  t_last_error.clear();
  const int rc = form_factor_host(m, n, A_mod, V, false);
  if (rc != DDCSVD_OK) {
    fprintf(stderr, "form_v_par: %s (%s)\n", ddcsvd_status_string(rc), ddcsvd_last_error());
    if (V && n > 0) V[0] = __builtin_nan("");
  }
}

}  // extern "C"
