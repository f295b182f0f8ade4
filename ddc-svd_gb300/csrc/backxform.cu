// backxform.cu -- stage 5: back-transformation U = Q_B [Y; 0], V = P_B X.
//
// Replaces multU / multV (bidiag_par.c:990-1095) and the transpose they rely
// on (svd_gpu.c:103, matrix_helper.c:166-174).  multV indexes A^T with the
// wrong leading dimension for m != n; here the right reflectors are read with
// their true layout.
//
// Blocked (BLOCKED modes): consecutive reflectors (kWY = 64 on the FP32 CUDA
// cores, kWYT = 128 on tcgen05) are aggregated into I - U T U^T (compact WY,
// T upper triangular) and applied per block, last block first:
// W1 = U^T C, then C -= U (T W1) -- on tcgen05 as two products with U T
// formed once per block.
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
__global__ void wy_tfactor_single_kernel(int bs, int j0, const float* __restrict__ tau, const float* __restrict__ G,
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

// ---------------------------------------------------------------- tensor-core path
// All reflectors of one side as an explicit column-major matrix Uc (column j
// = reflector j over the rows of C: zero above its unit entry at row j + side,
// the stored vector below, all zero when tau_j = 0).  Left reflectors are
// columns of W, right reflectors rows of W (transposed here through a 32 x 32
// shared-memory tile, so both reads and writes are coalesced).
__global__ void build_reflectors_kernel(int side, int rows_total, int nref, const float* __restrict__ W, int ldw,
                                        const float* __restrict__ tau, float* Uc, int ldu) {
  __shared__ float tile[32][33];  // [row][reflector]
  const int r0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    // side 0 reads W[r, j] along r; side 1 reads W[j, r] along j
    const int r = side == 0 ? r0 + threadIdx.x : r0 + k;
    const int j = side == 0 ? j0 + k : j0 + threadIdx.x;
    float v = 0.f;
    if (r < rows_total && j < nref && tau[j] != 0.f) {
      if (r == j + side) v = 1.f;
      else if (r > j + side) v = side == 0 ? W[r + (size_t)j * ldw] : W[j + (size_t)r * ldw];
    }
    if (side == 0) tile[threadIdx.x][k] = v;
    else tile[k][threadIdx.x] = v;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + threadIdx.x, j = j0 + k;
    if (r < ldu && j < nref) Uc[r + (size_t)j * ldu] = tile[threadIdx.x][k];
  }
}

// Offset (floats) of block b's U_b T_b in the packed UT array: block b covers
// rows [b NB, rows_total) and is stored row-major with NB columns.
template <int NB = kWY>
__host__ __device__ inline long long ut_offset(int b, int rows_total) {
  return (long long)NB * ((long long)b * rows_total - (long long)NB * b * (b - 1) / 2);
}

// WY preparation of every block b (reflectors j0 = b NB ... j0 + bs - 1,
// rows [j0, rows_total) of Uc), in four row- or entry-parallel kernels:
//   wy_gram_kernel     grid (block, row chunk): partial G = U^T U of a chunk
//   wy_gsum_kernel     grid (entries, block): G = sum of the chunk partials
//                      in chunk order, thread per entry
//   wy_tfactor_kernel  grid (block): the compact-WY factor T from G
//                      (T[l,l] = tau_l, T[0:l, l] = -tau_l T[0:l, 0:l] G[0:l, l])
//   wy_ut_kernel       grid (block, row chunk): UT = U T (row-major, ld NB)
// so that applying the block is C -= UT (U^T C) (or, with T^T, the
// transposed block of a QR factorisation).  A single CTA per block had cost
// 1.3 ms for an 8192-row block.  NB = 32 (QR panels) or 128 (QR super-blocks
// and the back-transformation: half the passes over C of 64-reflector blocks).
constexpr int kPrepRows = 32;    // rows per shared-memory tile
constexpr int kChunkRows = 512;  // rows per CTA of the chunked kernels (many blocks)
constexpr int kChunkRowsFew = 128;  // the same when a call has at most two blocks (QR panels / super-blocks)
__host__ __device__ inline int wy_chunk_rows(int nblk) { return nblk <= 2 ? kChunkRowsFew : kChunkRows; }
constexpr int kWYT = 128;        // reflectors per WY block of the tensor-core back-transformation

template <int NB>
__device__ __forceinline__ void wy_block_geom(int b, int rows_total, int nref, int& j0, int& bs, int& rows) {
  j0 = b * NB;
  bs = min(NB, nref - j0);
  rows = rows_total - j0;
}

template <int NB>
__device__ __forceinline__ void wy_load_tile(float (*sU)[NB + 1], const float* U, int ldu, int r0, int rend,
                                             int bs) {
  for (int idx = threadIdx.x; idx < kPrepRows * NB; idx += blockDim.x) {
    const int rr = idx & (kPrepRows - 1), c = idx / kPrepRows;
    const int r = r0 + rr;
    sU[rr][c] = (r < rend && c < bs) ? U[r + (size_t)c * ldu] : 0.f;
  }
}

// 256 threads as 16 x 16, each an (NB/16) x (NB/16) tile of G.
template <int NB>
__global__ void __launch_bounds__(256) wy_gram_kernel(int rows_total, int nref, const float* __restrict__ Uc, int ldu,
                                                      float* Gp, int nchunk, int chunk) {
  constexpr int R = NB / 16;
  __shared__ float sU[kPrepRows][NB + 1];
  int j0, bs, rows;
  wy_block_geom<NB>(blockIdx.x, rows_total, nref, j0, bs, rows);
  const int c0 = blockIdx.y * chunk;
  if (bs <= 0 || c0 >= rows) return;
  const int c1 = min(rows, c0 + chunk);
  const float* U = Uc + j0 + (size_t)j0 * ldu;
  const int t = threadIdx.x, ti = t & 15, tj = t >> 4;
  float acc[R][R];
#pragma unroll
  for (int a = 0; a < R; a++)
#pragma unroll
    for (int c = 0; c < R; c++) acc[a][c] = 0.f;
  for (int r0 = c0; r0 < c1; r0 += kPrepRows) {
    __syncthreads();
    wy_load_tile<NB>(sU, U, ldu, r0, c1, bs);
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kPrepRows; k++) {
      float x[R], y[R];
#pragma unroll
      for (int a = 0; a < R; a++) {
        x[a] = sU[k][R * ti + a];
        y[a] = sU[k][R * tj + a];
      }
#pragma unroll
      for (int a = 0; a < R; a++)
#pragma unroll
        for (int c = 0; c < R; c++) acc[a][c] += x[a] * y[c];
    }
  }
  float* G = Gp + ((size_t)blockIdx.x * nchunk + blockIdx.y) * NB * NB;
#pragma unroll
  for (int a = 0; a < R; a++)
#pragma unroll
    for (int c = 0; c < R; c++) G[(R * ti + a) + (size_t)(R * tj + c) * NB] = acc[a][c];
}

// G of every block: the chunk partials of each entry added in chunk order
// (thread per entry; grid (NB^2 / 256, blocks)).
template <int NB>
__global__ void __launch_bounds__(256) wy_gsum_kernel(int rows_total, int nref, const float* __restrict__ Gp,
                                                      int nchunk, int chunk, float* G) {
  int j0, bs, rows;
  wy_block_geom<NB>(blockIdx.y, rows_total, nref, j0, bs, rows);
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (bs <= 0 || rows <= 0 || idx >= NB * NB) return;
  const int nc = ceil_div(rows, chunk);
  const float* src = Gp + (size_t)blockIdx.y * nchunk * NB * NB + idx;
  float g = 0.f;
  for (int s = 0; s < nc; s++) g += src[(size_t)s * NB * NB];
  G[(size_t)blockIdx.y * NB * NB + idx] = g;
}

// 4 * NB threads, four per row of T; sG and sT in dynamic shared memory
// (2 NB (NB + 1) floats).
template <int NB>
__global__ void __launch_bounds__(4 * NB) wy_tfactor_kernel(int rows_total, int nref, const float* __restrict__ tau,
                                                            const float* __restrict__ G, float* Tout, int transT) {
  extern __shared__ float wsm[];
  float(*sG)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(wsm);
  float(*sT)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(wsm + NB * (NB + 1));
  int j0, bs, rows;
  wy_block_geom<NB>(blockIdx.x, rows_total, nref, j0, bs, rows);
  if (bs <= 0 || rows <= 0) return;
  const int t = threadIdx.x;
  const float* Gb = G + (size_t)blockIdx.x * NB * NB;
  for (int idx = t; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, c = idx / NB;
    sG[r][c] = Gb[idx];
    sT[r][c] = 0.f;
  }
  __syncthreads();
  {  // column l from the finished columns 0..l-1; four threads per row
    const int row = t >> 2, part = t & 3;
    for (int l = 0; l < bs; l++) {
      float sum = 0.f;
      if (row < l)
        for (int k = row + part; k < l; k += 4) sum += sT[row][k] * sG[k][l];
      sum += __shfl_xor_sync(0xffffffffu, sum, 1);
      sum += __shfl_xor_sync(0xffffffffu, sum, 2);
      const float tl = tau[j0 + l];
      if (part == 0 && row < l) sT[row][l] = -tl * sum;
      if (t == 0) sT[l][l] = tl;
      __syncthreads();
    }
  }
  // T (or T^T for a block applied as a transpose) to global, [row + col * NB]
  float* T = Tout + (size_t)blockIdx.x * NB * NB;
  for (int idx = t; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, c = idx / NB;
    T[idx] = transT ? sT[c][r] : sT[r][c];
  }
}

// 256 threads in NB / 4 column groups of 4 columns and 1024 / NB row groups
// of NB / 32 rows (a 32-row tile): per k one broadcast load of U per row and
// one 16-byte load of T for 4 NB / 32 FMAs.  sU ([32][NB + 1]) and sT
// ([NB][NB], T[k][c]) in dynamic shared memory.
template <int NB>
__global__ void __launch_bounds__(256) wy_ut_kernel(int rows_total, int nref, const float* __restrict__ Uc, int ldu,
                                                    const float* __restrict__ Tin, float* UT, int chunk) {
  constexpr int CG = NB / 4;    // column groups
  constexpr int RPT = NB / 32;  // rows per thread
  static_assert(256 / CG * RPT == kPrepRows, "row groups must cover the tile");
  extern __shared__ __align__(16) float wsm[];
  float(*sU)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(wsm);
  float(*sT)[NB] = reinterpret_cast<float(*)[NB]>(wsm + kPrepRows * (NB + 1));
  int j0, bs, rows;
  wy_block_geom<NB>(blockIdx.x, rows_total, nref, j0, bs, rows);
  const int c0 = blockIdx.y * chunk;
  if (bs <= 0 || c0 >= rows) return;
  const int c1 = min(rows, c0 + chunk);
  const float* U = Uc + j0 + (size_t)j0 * ldu;
  float* out = UT + ut_offset<NB>(blockIdx.x, rows_total);
  const int t = threadIdx.x;
  const float* T = Tin + (size_t)blockIdx.x * NB * NB;
  for (int idx = t; idx < NB * NB; idx += blockDim.x) sT[idx % NB][idx / NB] = T[idx];
  const int cg = t % CG, rg = t / CG;
  for (int r0 = c0; r0 < c1; r0 += kPrepRows) {
    __syncthreads();
    wy_load_tile<NB>(sU, U, ldu, r0, c1, bs);
    __syncthreads();
    float4 acc[RPT];
#pragma unroll
    for (int a = 0; a < RPT; a++) acc[a] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k < NB; k++) {
      const float4 y = *reinterpret_cast<const float4*>(&sT[k][4 * cg]);
#pragma unroll
      for (int a = 0; a < RPT; a++) {
        const float x = sU[rg * RPT + a][k];
        acc[a].x += x * y.x;
        acc[a].y += x * y.y;
        acc[a].z += x * y.z;
        acc[a].w += x * y.w;
      }
    }
#pragma unroll
    for (int a = 0; a < RPT; a++) {
      const int r = r0 + rg * RPT + a;
      if (r < c1) reinterpret_cast<float4*>(out + (size_t)r * NB)[cg] = acc[a];
    }
  }
}

// Scratch of wy_prepare_all: chunk partials and the T factors.
template <int NB = kWY>
static size_t wy_scratch_floats(int rows_total, int nref) {
  const int nblk = ceil_div(std::max(nref, 1), NB);
  const int nchunk = ceil_div(std::max(rows_total, 1), wy_chunk_rows(nblk));
  return (size_t)nblk * nchunk * NB * NB + 2 * (size_t)nblk * NB * NB + 64;
}

template <int NB>
static int wy_prepare_all(ddcsvd_context* ctx, int rows_total, int nref, const float* Uc, int ldu, const float* tau,
                          float* UT, bool transT, float* scratch) {
  const int nblk = ceil_div(nref, NB);
  const int chunk = wy_chunk_rows(nblk);
  const int nchunk = ceil_div(rows_total, chunk);
  float* Gp = scratch;
  float* G = scratch + (size_t)nblk * nchunk * NB * NB;
  float* T = G + (size_t)nblk * NB * NB;
  const int tf_smem = 2 * NB * (NB + 1) * (int)sizeof(float);
  const int ut_smem = (kPrepRows * (NB + 1) + NB * NB) * (int)sizeof(float);
  DDC_CUDA_TRY(cudaFuncSetAttribute((const void*)wy_tfactor_kernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    tf_smem));
  DDC_CUDA_TRY(cudaFuncSetAttribute((const void*)wy_ut_kernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    ut_smem));
  wy_gram_kernel<NB><<<dim3(nblk, nchunk), 256, 0, ctx->stream>>>(rows_total, nref, Uc, ldu, Gp, nchunk, chunk);
  wy_gsum_kernel<NB><<<dim3(ceil_div(NB * NB, 256), nblk), 256, 0, ctx->stream>>>(rows_total, nref, Gp, nchunk,
                                                                                  chunk, G);
  wy_tfactor_kernel<NB><<<nblk, 4 * NB, tf_smem, ctx->stream>>>(rows_total, nref, tau, G, T, transT ? 1 : 0);
  wy_ut_kernel<NB><<<dim3(nblk, nchunk), 256, ut_smem, ctx->stream>>>(rows_total, nref, Uc, ldu, T, UT, chunk);
  count_launch(4);
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

// One block of at most kPanel reflectors (a QR panel: columns of Vp, unit
// lower trapezoidal, rows x nb): UT = Vp T (or Vp T^T), row-major with kPanel
// columns.  The 32-wide kernels compute only the panel's 32 x 32 Gram matrix
// and T (the 64-wide ones had cost 34 ms over the 256 panels of a
// 16384 x 8192 QR).
size_t wy_block_scratch_floats(int rows) { return wy_scratch_floats<kPanel>(rows, kPanel); }

int wy_prepare_block(ddcsvd_context* ctx, int rows, int nb, const float* Vp, int ldv, const float* tau, float* UT,
                     bool transT, float* scratch) {
  if (nb > kPanel || rows <= 0) return DDCSVD_ERR_ARG;
  return wy_prepare_all<kPanel>(ctx, rows, nb, Vp, ldv, tau, UT, transT, scratch);
}

// The same for a block of at most kWideWY reflectors (UT row-major with
// kWideWY columns): the far trailing update of a 128-column QR super-block.
size_t wy_wide_scratch_floats(int rows) { return wy_scratch_floats<kWYT>(rows, kWYT); }

int wy_prepare_wide(ddcsvd_context* ctx, int rows, int nb, const float* Vp, int ldv, const float* tau, float* UT,
                    bool transT, float* scratch) {
  static_assert(kWYT == kWideWY, "one wide WY width");
  if (nb > kWYT || rows <= 0) return DDCSVD_ERR_ARG;
  return wy_prepare_all<kWYT>(ctx, rows, nb, Vp, ldv, tau, UT, transT, scratch);
}

// C (rows_total x ncols) := H_0 ... H_{nref-1} C on tensor cores.  Per block,
// last first:  W1 = U_b^T C (stored K-major for the next product) and
// C -= UT_b W1.
void bx_plan(int rows_total, int nref, int ncols, GemmKind kind, Arena& a, BxPrepared* out) {
  constexpr int NB = kWYT;
  BxPrepared& w = *out;
  w.ldu = (int)round_up(rows_total, 32);
  const int nblk = ceil_div(std::max(nref, 1), NB);
  w.Uc = a.take<float>((size_t)w.ldu * std::max(nref, 1));
  w.UT = a.take<float>((size_t)ut_offset<NB>(nblk, rows_total) + 64);
  w.W1s = a.take<float>((size_t)NB * ncols + 64);
  w.wys = a.take<float>(wy_scratch_floats<NB>(rows_total, nref));
  w.sbytes = gemm_scratch_bytes(kind, ncols, NB, rows_total);
  w.sc = a.take<char>(w.sbytes);
}

int bx_prepare(ddcsvd_context* ctx, int side, int rows_total, int nref, const float* W, int ldw, const float* tau,
               const BxPrepared& w) {
  constexpr int NB = kWYT;
  if (nref <= 0) return DDCSVD_OK;
  build_reflectors_kernel<<<dim3(ceil_div(w.ldu, 32), ceil_div(nref, 32)), dim3(32, 8), 0, ctx->stream>>>(
      side, rows_total, nref, W, ldw, tau, w.Uc, w.ldu);
  count_launch();
  DDC_TRY(wy_prepare_all<NB>(ctx, rows_total, nref, w.Uc, w.ldu, tau, w.UT, false, w.wys));
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

int bx_apply(ddcsvd_context* ctx, int rows_total, int nref, const BxPrepared& w, float* C, int ldc, int ncols,
             GemmKind kind) {
  constexpr int NB = kWYT;
  if (nref <= 0) return DDCSVD_OK;
  const int nblk = ceil_div(nref, NB);
  Arena scratch;
  scratch.base = w.sc;
  scratch.plan = false;
  scratch.cap = w.sbytes;
  for (int bi = nblk - 1; bi >= 0; bi--) {
    const int j0 = bi * NB;
    const int bs = std::min(NB, nref - j0);
    const int rows = rows_total - j0;
    if (rows <= 0 || bs <= 0) continue;
    // W1^T = C[j0:, :]^T U_b, stored as W1s[j + n * NB]
    DDC_TRY(gemm_tc_kmajor_t(ctx, kind, ncols, bs, rows, C, ldc, j0, w.Uc + (size_t)j0 * w.ldu, w.ldu, j0, w.W1s,
                             NB, 1.f, 0.f, &scratch));
    // C[j0:, :] -= UT_b W1
    DDC_TRY(gemm_tc_kmajor(ctx, kind, rows, ncols, bs, w.UT + ut_offset<NB>(bi, rows_total), NB, 0, w.W1s, NB, 0,
                           C + j0, ldc, -1.f, 1.f, &scratch));
  }
  return DDCSVD_OK;
}

static int apply_blocked_tc(ddcsvd_context* ctx, int side, int rows_total, int nref, const float* W, int ldw,
                            const float* tau, float* C, int ldc, int ncols, GemmKind kind, Arena& a,
                            bool plan_only) {
  BxPrepared w;
  bx_plan(rows_total, nref, ncols, kind, a, &w);
  if (plan_only) return DDCSVD_OK;
  DDC_TRY(bx_prepare(ctx, side, rows_total, nref, W, ldw, tau, w));
  return bx_apply(ctx, rows_total, nref, w, C, ldc, ncols, kind);
}

static int apply_blocked(ddcsvd_context* ctx, int side, int rows_total, int nref, const float* W,
                         int ldw, const float* tau, float* C, int ldc, int ncols, GemmKind kind,
                         Arena& a, bool plan_only) {
  const bool tc = (kind != GEMM_SIMT);
  if (tc) return apply_blocked_tc(ctx, side, rows_total, nref, W, ldw, tau, C, ldc, ncols, kind, a, plan_only);
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
    wy_tfactor_single_kernel<<<1, kWY, 0, ctx->stream>>>(bs, j0, tau, G, T);
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

// ---------------------------------------------------------------- explicit factors (FP64)
// Columns of the orthogonal factors of A = U B V^T from the reference's
// normalised reflectors (H = I - 2 v v^T, ||v|| = 1, as bidiag_par leaves
// them in A_mod), one warp per column in FP64, in the reference's order:
//   U[:, i] = H_0 ... H_{js(i)} e_i,  js(i) = min(i, mn - 1)        (form_u_par, bidiag_par.c:877-929)
//   V[:, i] = G_0 ... G_{js(i)} e_i,  js(i) = min(i - 1, nref - 1)  (form_v_par, bidiag_par.c:932-988)
// Reflectors beyond js(i) act on rows where e_i is zero and are skipped, as
// in the reference.  Right reflector j is row j of A_mod from column j + 1,
// read from a transposed copy (RT[k + j * n] = A_mod[j + k * m]).
__global__ void form_factor_kernel(int rows, int nref, int shift, const double* __restrict__ R, int ldr,
                                   double* Q) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < rows; i += nwarps) {
    double* col = Q + (size_t)i * rows;
    for (int k = lane; k < rows; k += 32) col[k] = (k == i) ? 1.0 : 0.0;
    __syncwarp();
    const int js = min(i - shift, nref - 1);
    for (int j = js; j >= 0; j--) {
      const double* v = R + (size_t)j * ldr;  // v(k) = v[k], k >= j + shift
      double sdot = 0.0;
      for (int k = j + shift + lane; k < rows; k += 32) sdot += col[k] * v[k];
      sdot = warp_sum(sdot);
      for (int k = j + shift + lane; k < rows; k += 32) col[k] -= 2.0 * v[k] * sdot;
      __syncwarp();
    }
  }
}

__global__ void transpose_f64_kernel(int rows, int cols, const double* __restrict__ A, int lda, double* AT,
                                     int ldat) {
  __shared__ double tile[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int r = r0 + threadIdx.x, c = c0 + k;
    tile[k][threadIdx.x] = (r < rows && c < cols) ? A[r + (size_t)c * lda] : 0.0;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int c = c0 + threadIdx.x, r = r0 + k;
    if (r < rows && c < cols) AT[c + (size_t)r * ldat] = tile[threadIdx.x][k];
  }
}

int form_factor_f64(ddcsvd_context* ctx, int m, int n, const double* dA, bool left, double* dQ, double* scratch) {
  const int mn = std::min(m, n);
  if (left) {
    form_factor_kernel<<<std::min(ceil_div(m, 8), 8 * ctx->num_sms), 256, 0, ctx->stream>>>(m, mn, 0, dA, m, dQ);
    count_launch();
  } else {
    const int nref = (m < n) ? mn : mn - 1;
    // RT (n x n): RT[k + j * n] = A_mod[j + k * m] for the first min(m, n) rows j
    transpose_f64_kernel<<<dim3(ceil_div(mn, 32), ceil_div(n, 32)), dim3(32, 8), 0, ctx->stream>>>(mn, n, dA, m,
                                                                                                  scratch, n);
    form_factor_kernel<<<std::min(ceil_div(n, 8), 8 * ctx->num_sms), 256, 0, ctx->stream>>>(n, nref, 1, scratch, n,
                                                                                         dQ);
    count_launch(2);
  }
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
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
