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
                          float* UT, bool transT, float* scratch, bool with_ut = true) {
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
  if (with_ut) wy_ut_kernel<NB><<<dim3(nblk, nchunk), 256, ut_smem, ctx->stream>>>(rows_total, nref, Uc, ldu, T, UT, chunk);
  count_launch(with_ut ? 4 : 3);
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
// ---------------------------------------------------------------- 256-reflector blocks
// The tensor-core back-transformation applies pairs of 128-reflector blocks
// (a = reflectors j0 .. j0+127, b = the next 128) as one WY block of 256:
//   Q_a Q_b = I - [U_a U_b] T [U_a U_b]^T,  T = [T_a, T_ab; 0, T_b],
//   T_ab = -T_a (U_a^T U_b) T_b
// (the standard concatenation of compact-WY factors), so that every pass
// over C does twice the reflectors: K = 256 in C -= (U T) W1 and N = 256 in
// W1^T = C^T U.  The 128-wide T factors come from wy_prepare_all; the kernels
// below add the cross Gram matrix U_a^T U_b, T_ab, and U T row-major with 256
// columns.
constexpr int kPairNB = 2 * kWYT;

__host__ __device__ inline long long ut2_offset(int p, int rows_total) {
  return (long long)kPairNB * ((long long)p * rows_total - (long long)kPairNB * p * (p - 1) / 2);
}

__device__ __forceinline__ void pair_geom(int p, int nref, int& j0, int& bsa, int& bsb) {
  j0 = p * kPairNB;
  bsa = min(kWYT, nref - j0);
  bsb = max(0, min(kWYT, nref - j0 - kWYT));
}

// Partial X = U_a^T U_b over a chunk of rows (grid (pair, chunk)); rows
// below j0 + 128 contribute nothing (U_b is zero there).
__global__ void __launch_bounds__(256) wy_xgram_kernel(int rows_total, int nref, const float* __restrict__ Uc,
                                                       int ldu, float* Xp, int nchunk, int chunk) {
  constexpr int NB = kWYT, R = NB / 16;
  __shared__ float sA[kPrepRows][NB + 1];
  __shared__ float sB[kPrepRows][NB + 1];
  int j0, bsa, bsb;
  pair_geom(blockIdx.x, nref, j0, bsa, bsb);
  const int jb = j0 + kWYT;
  const int c0 = jb + blockIdx.y * chunk;
  const int t = threadIdx.x, ti = t & 15, tj = t >> 4;
  float acc[R][R];
#pragma unroll
  for (int x = 0; x < R; x++)
#pragma unroll
    for (int y = 0; y < R; y++) acc[x][y] = 0.f;
  if (bsb > 0 && c0 < rows_total) {
    const int c1 = min(rows_total, c0 + chunk);
    const float* Ua = Uc + (size_t)j0 * ldu;
    const float* Ub = Uc + (size_t)jb * ldu;
    for (int r0 = c0; r0 < c1; r0 += kPrepRows) {
      __syncthreads();
      wy_load_tile<NB>(sA, Ua, ldu, r0, c1, bsa);
      wy_load_tile<NB>(sB, Ub, ldu, r0, c1, bsb);
      __syncthreads();
#pragma unroll 4
      for (int k = 0; k < kPrepRows; k++) {
        float x[R], y[R];
#pragma unroll
        for (int q = 0; q < R; q++) {
          x[q] = sA[k][R * ti + q];
          y[q] = sB[k][R * tj + q];
        }
#pragma unroll
        for (int q = 0; q < R; q++)
#pragma unroll
          for (int c = 0; c < R; c++) acc[q][c] += x[q] * y[c];
      }
    }
  }
  float* X = Xp + ((size_t)blockIdx.x * nchunk + blockIdx.y) * NB * NB;
#pragma unroll
  for (int q = 0; q < R; q++)
#pragma unroll
    for (int c = 0; c < R; c++) X[(R * ti + q) + (size_t)(R * tj + c) * NB] = acc[q][c];
}

// X of every pair: the chunk partials added in chunk order (thread per entry).
__global__ void __launch_bounds__(256) wy_xsum_kernel(const float* __restrict__ Xp, int nchunk, float* X) {
  constexpr int NB = kWYT;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= NB * NB) return;
  const float* src = Xp + (size_t)blockIdx.y * nchunk * NB * NB + idx;
  float g = 0.f;
  for (int c = 0; c < nchunk; c++) g += src[(size_t)c * NB * NB];
  X[(size_t)blockIdx.y * NB * NB + idx] = g;
}

// T_ab = -T_a X T_b for one pair per CTA (256 threads, each an 8 x 8 tile of
// the 128 x 128 result); sTa, sX and sTb in dynamic shared memory.
__global__ void __launch_bounds__(256) wy_tmerge_kernel(int nref, const float* __restrict__ T, const float* __restrict__ X,
                                                        float* Tab) {
  constexpr int NB = kWYT, R = NB / 16;
  extern __shared__ float wsm[];
  float(*sTa)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(wsm);
  float(*sX)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(wsm + NB * (NB + 1));
  float(*sTb)[NB + 1] = reinterpret_cast<float(*)[NB + 1]>(wsm + 2 * NB * (NB + 1));
  const int p = blockIdx.x, t = threadIdx.x, ti = t & 15, tj = t >> 4;
  int j0, bsa, bsb;
  pair_geom(p, nref, j0, bsa, bsb);
  float* out = Tab + (size_t)p * NB * NB;
  if (bsb <= 0) {
    for (int idx = t; idx < NB * NB; idx += blockDim.x) out[idx] = 0.f;
    return;
  }
  const float* Ta = T + (size_t)(2 * p) * NB * NB;  // [r + c NB]
  const float* Tb = T + (size_t)(2 * p + 1) * NB * NB;
  const float* Xg = X + (size_t)p * NB * NB;
  for (int idx = t; idx < NB * NB; idx += blockDim.x) {
    const int r = idx % NB, c = idx / NB;
    sTa[r][c] = Ta[idx];
    sX[r][c] = Xg[idx];
    sTb[r][c] = Tb[idx];
  }
  __syncthreads();
  float acc[R][R];
  // Y = X T_b
#pragma unroll
  for (int q = 0; q < R; q++)
#pragma unroll
    for (int c = 0; c < R; c++) acc[q][c] = 0.f;
  for (int k = 0; k < NB; k++) {
    float x[R], y[R];
#pragma unroll
    for (int q = 0; q < R; q++) {
      x[q] = sX[R * ti + q][k];
      y[q] = sTb[k][R * tj + q];
    }
#pragma unroll
    for (int q = 0; q < R; q++)
#pragma unroll
      for (int c = 0; c < R; c++) acc[q][c] += x[q] * y[c];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < R; q++)
#pragma unroll
    for (int c = 0; c < R; c++) sX[R * ti + q][R * tj + c] = acc[q][c];
  __syncthreads();
  // T_ab = -T_a Y
#pragma unroll
  for (int q = 0; q < R; q++)
#pragma unroll
    for (int c = 0; c < R; c++) acc[q][c] = 0.f;
  for (int k = 0; k < NB; k++) {
    float x[R], y[R];
#pragma unroll
    for (int q = 0; q < R; q++) {
      x[q] = sTa[R * ti + q][k];
      y[q] = sX[k][R * tj + q];
    }
#pragma unroll
    for (int q = 0; q < R; q++)
#pragma unroll
      for (int c = 0; c < R; c++) acc[q][c] += x[q] * y[c];
  }
#pragma unroll
  for (int q = 0; q < R; q++)
#pragma unroll
    for (int c = 0; c < R; c++) out[(R * ti + q) + (size_t)(R * tj + c) * NB] = -acc[q][c];
}

// UT of every pair, row-major with 256 columns over rows [j0, rows_total):
// half 0 (columns 0-127) = U_a T_a, half 1 = U_a T_ab + U_b T_b, i.e. the
// rows of [U_a U_b] times the half's 256 x 128 slice of the pair's T (grid
// (pair, row chunk, half); sU [32][257] and the slice in dynamic shared
// memory).  256 threads in 32 column groups of 4 columns and 8 row groups of
// 4 rows of a 32-row tile, as wy_ut_kernel.
__global__ void __launch_bounds__(256) wy_ut2_kernel(int rows_total, int nref, const float* __restrict__ Uc, int ldu,
                                                     const float* __restrict__ T, const float* __restrict__ Tab,
                                                     float* UT2, int chunk) {
  constexpr int NB = kWYT, KP = kPairNB, CG = NB / 4, RPT = 4;
  static_assert(256 / CG * RPT == kPrepRows, "row groups must cover the tile");
  extern __shared__ __align__(16) float wsm[];
  float(*sU)[KP + 1] = reinterpret_cast<float(*)[KP + 1]>(wsm);
  float(*sT)[NB] = reinterpret_cast<float(*)[NB]>(wsm + kPrepRows * (KP + 1));
  const int p = blockIdx.x, half = blockIdx.z, t = threadIdx.x;
  int j0, bsa, bsb;
  pair_geom(p, nref, j0, bsa, bsb);
  if (half == 1 && bsb <= 0) return;
  const int c0 = j0 + blockIdx.y * chunk;
  if (c0 >= rows_total) return;
  const int c1 = min(rows_total, c0 + chunk);
  const int kin = (half == 0) ? NB : KP;  // inner dimension of this half
  // the half's slice of T: rows 0-127 T_a (half 0) or T_ab (half 1), rows 128-255 T_b (half 1)
  const float* Ta = T + (size_t)(2 * p) * NB * NB;
  const float* Tb = T + (size_t)(2 * p + 1) * NB * NB;
  const float* Tx = Tab + (size_t)p * NB * NB;
  for (int idx = t; idx < kin * NB; idx += blockDim.x) {
    const int k = idx % kin, c = idx / kin;
    float v;
    if (half == 0) v = Ta[k + (size_t)c * NB];
    else v = (k < NB) ? Tx[k + (size_t)c * NB] : Tb[(k - NB) + (size_t)c * NB];
    sT[k][c] = v;
  }
  const int cg = t % CG, rg = t / CG;
  float* out = UT2 + ut2_offset(p, rows_total);
  for (int r0 = c0; r0 < c1; r0 += kPrepRows) {
    __syncthreads();
    for (int idx = t; idx < kPrepRows * kin; idx += blockDim.x) {
      const int rr = idx & (kPrepRows - 1), k = idx / kPrepRows;
      const int r = r0 + rr;
      const int bs = (k < NB) ? bsa : bsb;
      const int col = j0 + k;  // reflector index (b's columns follow a's)
      sU[rr][k] = (r < c1 && (k % NB) < bs) ? Uc[r + (size_t)col * ldu] : 0.f;
    }
    __syncthreads();
    float4 acc[RPT];
#pragma unroll
    for (int q = 0; q < RPT; q++) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int k = 0; k < kin; k++) {
      const float4 y = *reinterpret_cast<const float4*>(&sT[k][4 * cg]);
#pragma unroll
      for (int q = 0; q < RPT; q++) {
        const float x = sU[rg * RPT + q][k];
        acc[q].x += x * y.x;
        acc[q].y += x * y.y;
        acc[q].z += x * y.z;
        acc[q].w += x * y.w;
      }
    }
#pragma unroll
    for (int q = 0; q < RPT; q++) {
      const int r = r0 + rg * RPT + q;
      if (r < c1) reinterpret_cast<float4*>(out + (size_t)(r - j0) * KP + half * NB)[cg] = acc[q];
    }
  }
}

static size_t ut2_smem_bytes() { return sizeof(float) * ((size_t)kPrepRows * (kPairNB + 1) + (size_t)kPairNB * kWYT); }

void bx_plan(int rows_total, int nref, int ncols, GemmKind kind, Arena& a, BxPrepared* out) {
  constexpr int NB = kWYT;
  BxPrepared& w = *out;
  w.ldu = (int)round_up(rows_total, 32);
  const int npair = ceil_div(std::max(nref, 1), kPairNB);
  const int nchunk = ceil_div(std::max(rows_total, 1), kChunkRows);
  w.Uc = a.take<float>((size_t)w.ldu * std::max(nref, 1));
  w.UT = a.take<float>((size_t)ut2_offset(npair, rows_total) + 64);
  w.W1s = a.take<float>((size_t)kPairNB * ncols + 64);
  // wy_prepare_all's scratch (Gram partials, G, T of the 128-blocks), then
  // the pairs' cross-Gram partials, X and T_ab
  w.wys = a.take<float>(wy_scratch_floats<NB>(rows_total, nref) + (size_t)npair * (nchunk + 2) * NB * NB + 64);
  w.sbytes = gemm_scratch_bytes(kind, ncols, kPairNB, rows_total);
  w.sc = a.take<char>(w.sbytes);
}

int bx_prepare(ddcsvd_context* ctx, int side, int rows_total, int nref, const float* W, int ldw, const float* tau,
               const BxPrepared& w) {
  constexpr int NB = kWYT;
  if (nref <= 0) return DDCSVD_OK;
  build_reflectors_kernel<<<dim3(ceil_div(w.ldu, 32), ceil_div(nref, 32)), dim3(32, 8), 0, ctx->stream>>>(
      side, rows_total, nref, W, ldw, tau, w.Uc, w.ldu);
  count_launch();
  // T of every 128-block (wy_prepare_all's layout: Gram partials, G, then T)
  DDC_TRY(wy_prepare_all<NB>(ctx, rows_total, nref, w.Uc, w.ldu, tau, nullptr, false, w.wys, false));
  const int nblk = ceil_div(nref, NB);
  const int nchunk_g = ceil_div(rows_total, wy_chunk_rows(nblk));
  const float* T = w.wys + (size_t)nblk * nchunk_g * NB * NB + (size_t)nblk * NB * NB;
  const int npair = ceil_div(nref, kPairNB);
  const int nchunk = ceil_div(rows_total, kChunkRows);
  float* Xp = w.wys + wy_scratch_floats<NB>(rows_total, nref);
  float* X = Xp + (size_t)npair * nchunk * NB * NB;
  float* Tab = X + (size_t)npair * NB * NB;
  wy_xgram_kernel<<<dim3(npair, nchunk), 256, 0, ctx->stream>>>(rows_total, nref, w.Uc, w.ldu, Xp, nchunk,
                                                                kChunkRows);
  wy_xsum_kernel<<<dim3(ceil_div(NB * NB, 256), npair), 256, 0, ctx->stream>>>(Xp, nchunk, X);
  const int tm_smem = 3 * NB * (NB + 1) * (int)sizeof(float);
  DDC_CUDA_TRY(cudaFuncSetAttribute((const void*)wy_tmerge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    tm_smem));
  wy_tmerge_kernel<<<npair, 256, tm_smem, ctx->stream>>>(nref, T, X, Tab);
  const int ut_smem = (int)ut2_smem_bytes();
  DDC_CUDA_TRY(cudaFuncSetAttribute((const void*)wy_ut2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    ut_smem));
  wy_ut2_kernel<<<dim3(npair, nchunk, 2), 256, ut_smem, ctx->stream>>>(rows_total, nref, w.Uc, w.ldu, T, Tab, w.UT,
                                                                      kChunkRows);
  count_launch(4);
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

int bx_apply(ddcsvd_context* ctx, int rows_total, int nref, const BxPrepared& w, float* C, int ldc, int ncols,
             GemmKind kind) {
  if (nref <= 0) return DDCSVD_OK;
  const int npair = ceil_div(nref, kPairNB);
  Arena scratch;
  scratch.base = w.sc;
  scratch.plan = false;
  scratch.cap = w.sbytes;
  for (int p = npair - 1; p >= 0; p--) {
    const int j0 = p * kPairNB;
    const int bs = std::min(kPairNB, nref - j0);
    const int rows = rows_total - j0;
    if (rows <= 0 || bs <= 0) continue;
    // W1^T = C[j0:, :]^T U_p, stored as W1s[j + n * 256]
    DDC_TRY(gemm_tc_kmajor_t(ctx, kind, ncols, bs, rows, C, ldc, j0, w.Uc + (size_t)j0 * w.ldu, w.ldu, j0, w.W1s,
                             kPairNB, 1.f, 0.f, &scratch));
    // C[j0:, :] -= UT_p W1
    DDC_TRY(gemm_tc_kmajor(ctx, kind, rows, ncols, bs, w.UT + ut2_offset(p, rows_total), kPairNB, 0, w.W1s, kPairNB,
                           0, C + j0, ldc, -1.f, 1.f, &scratch));
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
