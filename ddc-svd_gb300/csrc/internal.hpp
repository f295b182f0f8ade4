// internal.hpp -- declarations shared by the translation units of libddcsvd.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include <functional>

#include "common.cuh"

struct ddcsvd_context {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;  // opt-in shared memory per block (bytes)
  int tail_cluster = -1;  // cluster size of the bidiagonalisation tail (0 = none, -1 = not yet probed)
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // the handle's second stream: work that needs nothing from the stages
  // running on `stream` meanwhile (the back-transformation's WY preparation
  // runs there during stages 2-4), forked and joined through two events
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // set by the host-buffer API: once the pipeline's second output (V, or U
  // of a wide input) is final it records v_ready, makes the side stream wait
  // for it and calls v_copy to queue that output's copy to the host there,
  // so the copy overlaps the rest of the back-transformation
  cudaEvent_t v_ready = nullptr;
  std::function<cudaError_t(cudaStream_t)> v_copy;
  bool v_copy_started = false;
  // device workspace (grown on demand, reused across calls)
  void* ws = nullptr;
  size_t ws_bytes = 0;
  // pinned host staging for the host-buffer entry points
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  // status word (device) and its pinned mirror
  ddcsvd::DevStatus* d_status = nullptr;
  ddcsvd::DevStatus* h_status = nullptr;
  // optional stage timing
  bool timing = false;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  float stage_ms[4] = {0, 0, 0, 0};
  // optional per-kernel-class timing (event pairs around launches)
  std::vector<cudaEvent_t> kev;       // pool, pairs
  std::vector<int> kcat;              // category of each recorded pair
  int kused = 0;
  float kern_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int kern_n[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  // launch-configuration knobs (ddcsvd_set_tuning / ddcsvd_autotune_*); none
  // of them changes the arithmetic beyond the summation order of split-K and
  // of the D&C lane groups
  int tune[8] = {16, 0, 512, 1, 8, 2, 1, 512};
  // the handle's own stream-ordered memory pool (per-call buffers: host-API
  // staging, QR-path blocks, aligned U/V copies); it keeps what it reserved
  // between calls (release threshold unlimited), so a repeated call maps no
  // new pages; ddcsvd_release_workspace trims it
  cudaMemPool_t pool = nullptr;
  // limits (ddcsvd_set_limits): FP64 secular iterations per root, the
  // wall-clock limit of device waits (us, 0 = the built-in 4 s), the
  // workspace budget (bytes, 0 = none), and the fault-injection count of
  // missing grid-barrier arrivals
  int sec_maxit = 80;
  unsigned wait_us = 0;
  size_t ws_cap = 0;
  unsigned barrier_extra = 0;
  // set while an SVD of the R factor runs inside the tall-matrix path
  bool nested = false;
  std::mutex mu;
};

namespace ddcsvd {
// A per-call device buffer from the handle's pool, ordered on its stream
// (released with cudaFreeAsync on the same stream).
template <typename T>
inline cudaError_t pool_alloc(ddcsvd_context* c, T** p, size_t bytes) {
  return cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), bytes, c->pool, c->stream);
}

enum TuneKnob {
  TK_SPLITK_MAX = 0,     // cap on split-K pieces of the GEMMs (1 = no split)
  TK_TC_BN = 1,          // tensor-core tile width: 0 = by N (64 if N <= 64 else 128), 64 = always 64
  TK_BATCH_THREADS = 2,  // batched stage-1 CTA size (256 or 512)
  TK_BATCH_SMEM_FULL = 3,// 1: batched stage-1 problems resident up to the opt-in limit, 0: up to 24K entries
  TK_DC_TERMS = 4,       // D&C: secular-sum terms per lane that size the lane groups (2..32)
  TK_TALL_QR = 5,        // QR first for m >= 2n: 0 never, 1 always, 2 when the matrix exceeds 64M entries
  TK_PANEL_FUSED = 6,    // panel kernel: 1 one read of the trailing block per column (<= 8192 rows), 0 two GEMVs
  TK_PANEL_TAIL = 7,     // most columns left to the thread-block-cluster tail (0: never)
  TK_COUNT = 8
};
}  // namespace ddcsvd

namespace ddcsvd {

// Bump allocator over the context workspace.  `plan` mode only counts.
struct Arena {
  char* base = nullptr;
  size_t off = 0;
  bool plan = true;
  size_t cap = 0;  // capacity when used as a fixed scratch region (0 = unchecked)
  template <typename T>
  T* take(size_t count) {
    off = (size_t)round_up((long long)off, 256);
    T* p = plan ? nullptr : reinterpret_cast<T*>(base + off);
    off += count * sizeof(T);
    return p;
  }
};

// Kernel classes for ddcsvd_get_kernel_times.
enum KernelClass { KC_BIDIAG = 0, KC_TRAIL_GEMM = 1, KC_DC = 2, KC_VECTORS = 3, KC_BACKXFORM = 4, KC_QR = 5 };
void ktimer_begin(ddcsvd_context* ctx, int cls);  // no-ops unless timing is on
void ktimer_end(ddcsvd_context* ctx);
void ktimer_collect(ddcsvd_context* ctx);        // after a stream sync

int ensure_workspace(ddcsvd_context* ctx, size_t bytes);
int ensure_pinned(ddcsvd_context* ctx, size_t bytes);
int check_status(ddcsvd_context* ctx, const char* stage);  // syncs the stream
int reset_status(ddcsvd_context* ctx);

// ---------------------------------------------------------------- GEMM back ends
enum GemmKind { GEMM_SIMT = 0, GEMM_TF32X3 = 1, GEMM_BF16X3 = 2, GEMM_TF32X6 = 3 };

// Operand descriptor: element (r, c) of the logical matrix lives at
// p[r * rs + c * cs]; exactly one of rs / cs is 1.
struct Mat {
  const float* p;
  long long rs, cs;
};

// C(M x N, col-major, ldc) = beta * C + alpha * (A1 B1 + A2 B2), A_t: M x K_t, B_t: K_t x N.
// A2/B2 may be null (K2 = 0).
int gemm(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K1, Mat A1, Mat B1, int K2, Mat A2,
         Mat B2, float alpha, float beta, float* C, int ldc, Arena* scratch);
size_t gemm_scratch_bytes(GemmKind kind, int M, int N, int K);
bool tc_available(ddcsvd_context* ctx);
// Tensor-core GEMM on K-major operands: A row r at A + r*lda (K from a_koff),
// B column n at B + n*ldb (K from b_koff); koffs multiples of 4, ld*4 and the
// base pointers 16-byte aligned.
int gemm_tc_kmajor(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K, const float* A, long long lda,
                   int a_koff, const float* B, long long ldb, int b_koff, float* C, int ldc, float alpha,
                   float beta, Arena* scratch);
// The same with C stored transposed: element (r, c) of the M x N result at
// Ct[c + r * ldct].
int gemm_tc_kmajor_t(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K, const float* A, long long lda,
                     int a_koff, const float* B, long long ldb, int b_koff, float* Ct, int ldct, float alpha,
                     float beta, Arena* scratch);
// rows x (K1 + K2) K-major copy of two column-major blocks.
int pack_kmajor(ddcsvd_context* ctx, int rows, int K1, const float* P1, int ld1, int K2, const float* P2, int ld2,
                float* out, int ldo);

// ---------------------------------------------------------------- stage 1
struct BidiagWork {
  float *X, *Y, *VT;  // panel matrices (ldx = ldw, ldy = ldvt = ldn)
  int ldn;
  float *xcol, *xrow;
  float *colpart, *rowpart;
  GridBarrier* bar;
  unsigned* amax;  // max |a| of the input (bit pattern), for range scaling
  int P;  // CTAs of the cooperative launch
  char* gemm_scratch;
  float *Apk, *Bpk;  // K-major packed trailing-update operands (tensor-core modes)
  float* xpart;      // fused panel pass: P partial products x = A w (ld ldxp), or null
  int ldxp;
};
constexpr int kPanel = 32;       // bidiagonalisation panel width
constexpr int kFusedRows = 8192; // fused panel pass: rows (from the first staged float4) it covers
constexpr int kBidiagThreads = 512;
void plan_bidiag(Arena& a, int m, int n, int ldw, int P, GemmKind kind, BidiagWork* w);
int bidiag_blocked(ddcsvd_context* ctx, int m, int n, float* W, int ldw, float* d, float* e,
                   float* tauq, float* taup, BidiagWork& w, GemmKind kind, Arena* scratch);
int bidiag_plain(ddcsvd_context* ctx, int m, int n, float* W, int ldw, float* d, float* e,
                 float* tauq, float* taup, BidiagWork& w);
int bidiag_coop_ctas(ddcsvd_context* ctx, int m, int n);
// Columns from k0 on that the cluster tail can finish (0 = none: knob off,
// no co-schedulable cluster, or the trailing block does not fit), and the
// launch: the trailing block W[k0:m, k0:n] bidiagonalised on one cluster.
int bidiag_tail_columns(ddcsvd_context* ctx, int m, int n, int k0);
int bidiag_tail(ddcsvd_context* ctx, int m, int n, int k0, float* W, int ldw, float* d, float* e, float* tauq,
                float* taup);
// LAPACK-form reflectors -> the reference's normalised form, FP64 output (ld = m).
int export_reflectors(ddcsvd_context* ctx, int m, int n, const float* W, int ldw, const float* d,
                      const float* e, const float* tauq, const float* taup, double* A_out);

// ---------------------------------------------------------------- stage 2
// Host description of the D&C forest (one tree per unreduced block).
struct DcHost {
  int maxdepth = 0;
  int nnodes = 0, ndm = 0;
  // per-tree schedule (the tree kernel): trees, their depth segments, the
  // largest tree, and the offset of these arrays in `ints`
  int ntrees = 0, nseg = 0, maxtree = 0;
  size_t tree_off = 0;
  std::vector<int> ints;  // packed node table uploaded to the device
};
void dc_build_host(int N, const std::vector<int>& block_starts, DcHost& H, int terms_per_lane = 8);
size_t dc_max_ints(int N);
int dc_sigma(ddcsvd_context* ctx, int N, const double* b1, const double* b2, double* sigma,
             const DcHost* H, const int* dints, Arena& a, bool plan_only);

// Splits the N x N bidiagonal (host copies a[N], b[N]) at |b_i| <= 4 eps max|B|:
// zeroes those b_i (and b[N-1]), fills block_starts (ascending, ends with N)
// and, per row, the bounds of its block.
struct VecLayout;
int sort_values(ddcsvd_context* ctx, int N, const double* in, double* out, const VecLayout* L, Arena& a);
void split_bidiagonal(int N, double* a, double* b, double eps, std::vector<int>& block_starts,
                      int* blk_lo, int* blk_hi);

// ---------------------------------------------------------------- stages 3-4
struct VecLayout;
// sigma (slot order: ascending within each block) -> X, Y columns of every
// group in ascending order; sigma_sorted receives the sorted values (group
// ranges of slots).  `store` = sum over blocks of nb^2.
int bd_vectors(ddcsvd_context* ctx, int N, long long store, const double* a, const double* b,
               const double* sigma, const VecLayout* L, double* sigma_sorted, Arena& arena, bool plan_only);

// ---------------------------------------------------------------- stage 5
constexpr int kWY = 64;  // reflectors per WY block of the FP32 (SIMT) back-transformation; tcgen05 blocks take 128
// C (rows x ncols, ldc) := Q C with Q = H_0 ... H_{nref-1} (left reflectors in W columns).
int apply_left_reflectors(ddcsvd_context* ctx, int m, int nref, const float* W, int ldw,
                          const float* tauq, float* C, int ldc, int ncols, GemmKind kind,
                          bool plain, Arena& a, bool plan_only);
// C (n x ncols) := P C with P = G_0 ... G_{nref-1} (right reflectors in W rows).
int apply_right_reflectors(ddcsvd_context* ctx, int n, int nref, const float* W, int ldw,
                           const float* taup, float* C, int ldc, int ncols, GemmKind kind,
                           bool plain, Arena& a, bool plan_only);

// The tensor-core back-transformation in two halves: `bx_prepare` writes the
// reflectors as an explicit masked matrix and every 128-reflector block's
// T factor and U T (it reads only W and tau, so it may run on another stream
// while the singular vectors are computed); `bx_apply` then updates C with
// the prepared blocks, last block first.  side 0: left reflectors (columns
// of W, rows_total = m), 1: right reflectors (rows of W, rows_total = n).
struct BxPrepared {
  float* Uc = nullptr;
  float* UT = nullptr;
  float* W1s = nullptr;
  float* wys = nullptr;
  char* sc = nullptr;
  size_t sbytes = 0;
  int ldu = 0;
};
void bx_plan(int rows_total, int nref, int ncols, GemmKind kind, Arena& a, BxPrepared* out);  // buffers from `a`
int bx_prepare(ddcsvd_context* ctx, int side, int rows_total, int nref, const float* W, int ldw, const float* tau,
               const BxPrepared& w);
int bx_apply(ddcsvd_context* ctx, int rows_total, int nref, const BxPrepared& w, float* C, int ldc, int ncols,
             GemmKind kind);

// UT = Vp T (or Vp T^T) of one QR panel (nb <= kPanel reflectors), row-major with kPanel columns.
int wy_prepare_block(ddcsvd_context* ctx, int rows, int nb, const float* Vp, int ldv, const float* tau, float* UT,
                     bool transT, float* scratch);
size_t wy_block_scratch_floats(int rows);  // scratch of wy_prepare_block
constexpr int kWideWY = 128;  // reflectors per wide WY block (back-transformation, QR super-blocks)
// UT of at most kWideWY reflectors, row-major with kWideWY columns.
int wy_prepare_wide(ddcsvd_context* ctx, int rows, int nb, const float* Vp, int ldv, const float* tau, float* UT,
                    bool transT, float* scratch);
size_t wy_wide_scratch_floats(int rows);
// Householder QR of the m x n (m >= n) matrix W in place (R on and above the
// diagonal, reflectors below in LAPACK form, tau separate), tensor-core
// trailing updates; the input must be range-scaled (max|a| in [2^-40, 2^40]).
struct QrWork {
  float *Vp, *UT, *W1s, *part, *rowi, *wys;
  float *UTw, *W1w;  // far trailing update of a super-block (kWideWY reflectors)
  GridBarrier* bar;
  char* gemm_scratch;
  size_t gemm_scratch_bytes;
  int ldv, P;
};
void plan_qr(Arena& a, int m, int n, int P, GemmKind kind, QrWork* w);
int qr_blocked(ddcsvd_context* ctx, int m, int n, float* W, int ldw, float* tau, QrWork& w, GemmKind kind);
// Range scaling of an m x n matrix in place (power of two; scale 1 when max|a|
// is already in range); amax receives the bit pattern that range_scale uses.
int range_scale_matrix(ddcsvd_context* ctx, int m, int n, float* W, int ldw, unsigned* amax);
int range_unscale_vector(ddcsvd_context* ctx, int n, float* x, const unsigned* amax);

// Explicit U (m x m) or V (n x n) from the reference's FP64 reflector storage
// (device buffers; scratch: n * n doubles for V).
int form_factor_f64(ddcsvd_context* ctx, int m, int n, const double* dA, bool left, double* dQ, double* scratch);

}  // namespace ddcsvd
