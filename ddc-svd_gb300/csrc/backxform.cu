// backxform.cu -- stage 5: back-transformation U = Q_B [Y; 0], V = P_B X.
//
// Replaces multU / multV (bidiag_par.c:990-1095) and the transpose they rely
// on (svd_gpu.c:103, matrix_helper.c:166-174).  multV indexes A^T with the
// wrong leading dimension for m != n; here the right reflectors are read with
// their true layout.
//
// Blocked (BLOCKED modes): kWY consecutive reflectors are aggregated into
// I - U T U^T (compact WY, T upper triangular) and applied with three GEMMs
// per block, last block first:  W1 = U^T C,  W2 = T W1,  C -= U W2.
// The GEMMs run on the back end of the mode (FP32 CUDA cores or tcgen05).
//
// Plain (PLAIN_FP32): the reference's per-vector scheme -- every column of C
// is transformed by the reflectors one at a time (a dot product and an axpy
// per reflector, bidiag_par.c:1088-1094), one warp per column.
#include "internal.hpp"

namespace ddcsvd {

// Pack bs reflectors into a unit lower-trapezoidal m' x bs block (ld ldp).
// side 0 (left):  reflector j0+l is column j0+l of W from row j0+l, unit at
//                 row l of the block; block rows = W rows j0 ...
// side 1 (right): reflector j0+l is row j0+l of W from column j0+l+1, unit
//                 at row l of the block; block rows = positions j0+1 ...
// Block rows are shifted down by `sh` (< 4) zero rows so that the first row
// touched in C starts on a 16-byte boundary (tensor-memory-access rule).
__global__ void pack_reflectors_kernel(int side, int rows, int bs, int j0, int sh, const float* __restrict__ W,
                                       int ldw, const float* __restrict__ tau, float* P, int ldp) {
  const int l = blockIdx.y;
  for (int rp = blockIdx.x * blockDim.x + threadIdx.x; rp < rows + sh; rp += gridDim.x * blockDim.x) {
    const int r = rp - sh;
    float v;
    if (r < 0 || l >= bs || tau[j0 + l] == 0.f) v = 0.f;  // alignment pad / absent / identity reflector
    else if (r < l) v = 0.f;
    else if (r == l) v = 1.f;
    else v = side == 0 ? W[(j0 + r) + (size_t)(j0 + l) * ldw] : W[(j0 + l) + (size_t)(j0 + 1 + r) * ldw];
    P[rp + (size_t)l * ldp] = v;
  }
}

// T (bs x bs, col-major) from the Gram matrix G = U^T U:
//   T[l,l] = tau_l,  T[0:l, l] = -tau_l T[0:l, 0:l] G[0:l, l].
__global__ void wy_tfactor_kernel(int bs, int j0, const float* __restrict__ tau, const float* __restrict__ G,
                                  float* T) {
  __shared__ float sT[kWY][kWY + 1];
  __shared__ float sG[kWY][kWY + 1];
  __shared__ float col[kWY];
  const int t = threadIdx.x;
  for (int idx = t; idx < kWY * kWY; idx += blockDim.x) {
    const int r = idx % kWY, c = idx / kWY;
    sT[r][c] = 0.f;
    sG[r][c] = (r < bs && c < bs) ? G[r + (size_t)c * bs] : 0.f;
  }
  __syncthreads();
  for (int l = 0; l < bs; l++) {
    const float tl = tau[j0 + l];
    if (t < l) {
      float s = 0.f;
      for (int k = t; k < l; k++) s += sT[t][k] * sG[k][l];
      col[t] = -tl * s;
    }
    __syncthreads();
    if (t < l) sT[t][l] = col[t];
    if (t == 0) sT[l][l] = tl;
    __syncthreads();
  }
  for (int idx = t; idx < bs * bs; idx += blockDim.x) T[idx] = sT[idx % bs][idx / bs];
}

static int apply_blocked(ddcsvd_context* ctx, int side, int rows_total, int nref, const float* W,
                         int ldw, const float* tau, float* C, int ldc, int ncols, GemmKind kind,
                         Arena& a, bool plan_only) {
  const bool tc = (kind != GEMM_SIMT);
  const int ldp = (int)round_up(rows_total + 4, 32);
  float* Pk = a.take<float>((size_t)ldp * kWY);
  float* PkT = a.take<float>(tc ? (size_t)ldp * kWY : 16);
  float* G = a.take<float>(kWY * kWY);
  float* T = a.take<float>(kWY * kWY);
  float* W1 = a.take<float>((size_t)kWY * ncols);
  float* W2 = a.take<float>((size_t)kWY * ncols);
  const size_t sbytes = gemm_scratch_bytes(kind, std::max(rows_total, kWY), ncols, std::max(rows_total, kWY));
  char* sc = a.take<char>(sbytes);
  if (plan_only || nref <= 0) return DDCSVD_OK;
  Arena scratch;
  scratch.base = sc;
  scratch.plan = false;
  scratch.cap = sbytes;
  Mat none{nullptr, 0, 0};
  const int nblk = ceil_div(nref, kWY);
  for (int bi = nblk - 1; bi >= 0; bi--) {
    const int j0 = bi * kWY;
    const int bs = std::min(kWY, nref - j0);
    const int off = side == 0 ? j0 : j0 + 1;  // first row of C touched
    if (rows_total - off <= 0) continue;
    const int off_al = off & ~3, sh = off - off_al;
    const int rows = rows_total - off_al;  // block rows, including the sh zero rows on top
    dim3 g(std::min(ceil_div(rows, 256), 64), bs);
    pack_reflectors_kernel<<<g, 256, 0, ctx->stream>>>(side, rows - sh, bs, j0, sh, W, ldw, tau, Pk, ldp);
    count_launch();
    DDC_CUDA_TRY(cudaGetLastError());
    Mat UT{Pk, ldp, 1}, U{Pk, 1, ldp};
    // G = U^T U (bs x bs) and the triangular factor T
    DDC_TRY(gemm(ctx, GEMM_SIMT, bs, bs, rows, UT, U, 0, none, none, 1.f, 0.f, G, bs, &scratch));
    wy_tfactor_kernel<<<1, kWY, 0, ctx->stream>>>(bs, j0, tau, G, T);
    count_launch();
    float* Cb = C + off_al;
    if (!tc) {
      // W1 = U^T C (bs x ncols); W2 = T W1; C -= U W2
      DDC_TRY(gemm(ctx, kind, bs, ncols, rows, UT, Mat{Cb, 1, ldc}, 0, none, none, 1.f, 0.f, W1, bs, &scratch));
      DDC_TRY(gemm(ctx, GEMM_SIMT, bs, ncols, bs, Mat{T, 1, bs}, Mat{W1, 1, bs}, 0, none, none, 1.f, 0.f, W2, bs,
                   &scratch));
      DDC_TRY(gemm(ctx, kind, rows, ncols, bs, U, Mat{W2, 1, bs}, 0, none, none, -1.f, 1.f, Cb, ldc, &scratch));
    } else {
      // W1^T = C^T U (ncols x bs): C is already K-major for this product
      DDC_TRY(gemm_tc_kmajor(ctx, kind, ncols, bs, rows, C, ldc, off_al, Pk, ldp, 0, W1, ncols, 1.f, 0.f,
                             &scratch));
      // W2 = T W1 (bs x ncols, col-major with ld kWY: K-major rows, 16-byte aligned for any bs)
      DDC_TRY(gemm(ctx, GEMM_SIMT, bs, ncols, bs, Mat{T, 1, bs}, Mat{W1, ncols, 1}, 0, none, none, 1.f, 0.f, W2,
                   kWY, &scratch));
      // C -= U W2 with U packed K-major (rows x bs, ld kWY)
      DDC_TRY(pack_kmajor(ctx, rows, bs, Pk, ldp, 0, nullptr, 0, PkT, kWY));
      DDC_TRY(gemm_tc_kmajor(ctx, kind, rows, ncols, bs, PkT, kWY, 0, W2, kWY, 0, Cb, ldc, -1.f, 1.f, &scratch));
    }
  }
  return DDCSVD_OK;
}

// ---------------------------------------------------------------- plain path
__global__ void transpose_kernel(int rows, int cols, const float* __restrict__ A, int lda, float* AT,
                                 int ldat) {
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

// Each warp owns one column of C and applies reflectors nref-1 ... 0.
// Reflector j: vector R[j*ldr + off_j ...] of length rows_total - (j + shift),
// unit leading entry stored, scalar tau[j].
__global__ void __launch_bounds__(256) apply_plain_kernel(int rows_total, int nref, int shift,
                                                          const float* __restrict__ R, int ldr,
                                                          const float* __restrict__ tau, float* C,
                                                          int ldc, int ncols) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= ncols) return;
  float* col = C + (size_t)c * ldc;
  for (int j = nref - 1; j >= 0; j--) {
    const float tj = tau[j];
    if (tj == 0.f) continue;
    const int r0 = j + shift;
    const float* u = R + (size_t)j * ldr;
    float s = 0.f;
    for (int r = r0 + lane; r < rows_total; r += 32) s += u[r] * col[r];
    s = warp_sum(s);
    const float f = tj * s;
    for (int r = r0 + lane; r < rows_total; r += 32) col[r] -= f * u[r];
    __syncwarp();
  }
}

int apply_left_reflectors(ddcsvd_context* ctx, int m, int nref, const float* W, int ldw,
                          const float* tauq, float* C, int ldc, int ncols, GemmKind kind,
                          bool plain, Arena& a, bool plan_only) {
  if (!plain) {
    if (!plan_only) ktimer_begin(ctx, KC_BACKXFORM);
    int rc = apply_blocked(ctx, 0, m, nref, W, ldw, tauq, C, ldc, ncols, kind, a, plan_only);
    if (!plan_only) ktimer_end(ctx);
    return rc;
  }
  if (plan_only) return DDCSVD_OK;
  ktimer_begin(ctx, KC_BACKXFORM);
  // left reflector j is column j of W from row j (unit stored at W[j, j])
  apply_plain_kernel<<<ceil_div(ncols, 8), 256, 0, ctx->stream>>>(m, nref, 0, W, ldw, tauq, C, ldc, ncols);
  count_launch();
  ktimer_end(ctx);
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

int apply_right_reflectors(ddcsvd_context* ctx, int n, int nref, const float* W, int ldw,
                           const float* taup, float* C, int ldc, int ncols, GemmKind kind,
                           bool plain, Arena& a, bool plan_only) {
  if (!plain) {
    if (!plan_only) ktimer_begin(ctx, KC_BACKXFORM);
    int rc = apply_blocked(ctx, 1, n, nref, W, ldw, taup, C, ldc, ncols, kind, a, plan_only);
    if (!plan_only) ktimer_end(ctx);
    return rc;
  }
  const int ldt = (int)round_up(n, 32);
  float* WT = a.take<float>((size_t)ldt * n);
  if (plan_only || nref <= 0) return DDCSVD_OK;
  // WT = W[0:n, 0:n]^T so that right reflector j is column j of WT from row j+1
  ktimer_begin(ctx, KC_BACKXFORM);
  transpose_kernel<<<dim3(ceil_div(n, 32), ceil_div(n, 32)), dim3(32, 8), 0, ctx->stream>>>(n, n, W, ldw, WT, ldt);
  count_launch();
  apply_plain_kernel<<<ceil_div(ncols, 8), 256, 0, ctx->stream>>>(n, nref, 1, WT, ldt, taup, C, ldc, ncols);
  count_launch();
  ktimer_end(ctx);
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

}  // namespace ddcsvd
