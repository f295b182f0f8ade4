// batched.cu -- many independent SVDs of uneven sizes in one launch sequence.
//
// Stage 1 (bidiagonalisation) and stage 5 (back-transformation) run one CTA
// per problem: a persistent kernel pulls problems from an atomic work counter
// in decreasing-size order (host-sorted), keeps the problem in shared memory
// when it fits (global memory, L1/L2-resident, otherwise) and runs the
// reference's unblocked algorithm (bidiag.c:33-186; rank-1 left and right
// updates per step) with CTA-wide synchronisation only.  Stages 2-4 reuse the
// single-matrix machinery unchanged: every problem's bidiagonal becomes one
// or more trees of the D&C forest (one cooperative launch for the whole
// batch) and one output group of the vector stage.
//
// Problems with m < n are decomposed through A^T (U and V swap roles).
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "internal.hpp"
#include "prep.hpp"

namespace ddcsvd {

struct BatchTask {
  int m, n;      // oriented problem: m >= n
  int trans;     // 1 if the caller's matrix is n x m (decomposed as its transpose)
  int pad;
  long long offW;  // working copy (m x n, ld m)
  long long offD;  // first slot of the bidiagonal (sum of previous n)
  long long offA;  // caller's input
  long long offU;  // core left vectors (m x n, ld m) -> caller's U or V
  long long offV;  // core right vectors (n x n, ld n) -> caller's V or U
  long long offS;  // caller's sigma
};

constexpr int kBatchThreads = 256;        // back-transformation CTAs
constexpr int kBatchBidiagThreads = 512;  // bidiagonalisation CTAs (one per SM, whole problem in shared memory)

__device__ __forceinline__ float bsgn(float x) { return x < 0.f ? -1.f : 1.f; }

constexpr int kColRegs = 8;  // rows per lane of the register-held reflector (m - i <= 256)

// phase marks (trace builds): CTA 0; rows 0-63 the first 64 columns of its
// first problem (slots 0-4: column start, after each of the four barriers),
// rows 64-127 its problems in turn (slot 0 start, 1 end, 2 m, 3 n)
#ifdef DDCSVD_PHASE_TRACE
__device__ unsigned long long g_batch_trace[128 * 16];
#define BMARK(row, slot, val)                                                         \
  do {                                                                                \
    if (blockIdx.x == 0 && threadIdx.x == 0 && (row) < 128) g_batch_trace[(row) * 16 + (slot)] = (val); \
  } while (0)
#else
#define BMARK(row, slot, val) \
  do {                        \
  } while (0)
#endif

__device__ __forceinline__ int row_slices(int rows) { return rows <= 32 ? 1 : rows <= 64 ? 2 : rows <= 128 ? 4 : 8; }

// One pass of the batched column step over the trailing block (rows i.., at
// most 32 KR of them): a warp holds four columns in registers, forms their
// left dot products with u (u_i = 1, u_r = sq x_r), applies the left update,
// and with the new row-i values w_c (c >= i + 2) accumulates the partial
// right products sum_c a'_rc w_c of its rows into zs (its row of 256).  The
// four dot products are summed over the warp by a reduce-scatter (2 + 1
// shuffles leave each lane a partial of one column over 8 lanes, 3 more
// complete it) and a gather: 10 shuffles instead of 20.
template <int KR>
__device__ __forceinline__ void left_pass(float* M, int ld, int m, int n, int i, float tauq, float sq, float* zs,
                                          int lane, int wid, int nw) {
  const float* uc = M + (size_t)i * ld;
  const bool b16 = lane & 16, b8 = lane & 8;
  float u[KR], zp[KR];
#pragma unroll
  for (int k = 0; k < KR; k++) {
    const int r = i + lane + 32 * k;
    u[k] = (r < m) ? (r == i ? 1.f : uc[r] * sq) : 0.f;
    zp[k] = 0.f;
  }
  for (int c0 = i + 1 + 4 * wid; c0 < n; c0 += 4 * nw) {
    float a[4][KR];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = i + lane + 32 * k;
        a[q][k] = (c0 + q < n && r < m) ? M[r + (size_t)(c0 + q) * ld] : 0.f;
      }
    if (tauq != 0.f) {
      float w[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < KR; k++) s += u[k] * a[q][k];
        w[q] = s;
      }
      float e2[2];
#pragma unroll
      for (int q = 0; q < 2; q++)
        e2[q] = (b16 ? w[q + 2] : w[q]) + __shfl_xor_sync(0xffffffffu, b16 ? w[q] : w[q + 2], 16);
      float g = (b8 ? e2[1] : e2[0]) + __shfl_xor_sync(0xffffffffu, b8 ? e2[0] : e2[1], 8);
      g += __shfl_xor_sync(0xffffffffu, g, 4);
      g += __shfl_xor_sync(0xffffffffu, g, 2);
      g += __shfl_xor_sync(0xffffffffu, g, 1);
      // lane l holds the sum of column 2 b16 + b8
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float f = __shfl_sync(0xffffffffu, g, ((q >> 1) & 1) * 16 + (q & 1) * 8) * tauq;
#pragma unroll
        for (int k = 0; k < KR; k++) a[q][k] -= f * u[k];
        if (c0 + q < n) {
          float* col = M + (size_t)(c0 + q) * ld;
#pragma unroll
          for (int k = 0; k < KR; k++) {
            const int r = i + lane + 32 * k;
            if (r < m) col[r] = a[q][k];
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float wc = __shfl_sync(0xffffffffu, a[q][0], 0);  // new a_{i,c}
      if (c0 + q >= i + 2 && c0 + q < n)
#pragma unroll
        for (int k = 0; k < KR; k++) zp[k] += a[q][k] * wc;
    }
  }
#pragma unroll
  for (int k = 0; k < KR; k++) zs[wid * 32 * kColRegs + lane + 32 * k] = zp[k];
}

// Unblocked Golub-Kahan bidiagonalisation of M (m x n, ld, m >= n) by one CTA
// (the reference's bidiag_seq order, bidiag.c:33-186: left reflector and
// rank-1 update, then right reflector and rank-1 update, per column).
// Reflectors stay in M in LAPACK form (unit leading entry stored).  Norms are
// compensated FP32 sums and the reflector scalars FP32 (the caller keeps
// max|M| in [2^-40, 2^40]).  Warp 0 alone forms each reflector (norm,
// scalars, and for the right one the scaled row) and hands the scalars to
// the other warps through `sh` across the barrier that the update needs
// anyway: four CTA barriers per column.
//
// While the trailing rows fit the warps' registers (m - i <= 256) the left
// update and the right reflector's products share one pass over the block:
// a warp holds four columns of it in registers, updates them, and with the
// new row-i values w_c (c >= i + 2) accumulates sum_c a'_rc w_c for its
// rows; the right update then forms z_r = a'_{r,i+1} + sp * sum_c a'_rc w_c
// (v_{i+1} = 1, v_c = sp w_c) instead of a second pass of dot products.
// `zs` holds the warps' partial sums (blockDim.x / 32 rows of 256) and their
// totals (256 more).
__device__ void cta_bidiag(float* M, int ld, int m, int n, float* d, float* e, float* tq, float* tp,
                           float* vrow, float* zs, float* sh, int iend, bool trace = false) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
  constexpr int kZRows = 32 * kColRegs;
  float* zsum = zs + nw * kZRows;
  (void)trace;
  for (int i = 0; i < iend; i++) {
    const bool tr = trace && i < 64;
    (void)tr;
    BMARK(tr ? i : 999, 0, global_ns());
    // ---- left reflector from column i (warp 0)
    if (wid == 0) {
      const float x0 = M[i + (size_t)i * ld];
      FF s2{0.f, 0.f};
      for (int r = i + 1 + lane; r < m; r += 32) s2 = ff_add_sq(s2, M[r + (size_t)i * ld]);
      s2 = warp_sum_ff(s2);
      float alpha, tauq, sq;
      householder_ff(x0, s2, &alpha, &tauq, &sq);
      if (lane == 0) {
        d[i] = alpha;
        tq[i] = tauq;
        sh[0] = tauq;
        sh[1] = sq;
      }
    }
    __syncthreads();
    BMARK(tr ? i : 999, 1, global_ns());
    const float tauq = sh[0], sq = sh[1];
    if (i == n - 1) {  // last column: no update, only the reflector form
      if (t == 0) M[i + (size_t)i * ld] = 1.f;
      for (int r = i + 1 + t; r < m; r += blockDim.x) M[r + (size_t)i * ld] *= sq;
      break;
    }
    // ---- left update of columns > i (left_dotprods + left_update_mat).
    // The reflector is formed from the stored column as u_i = 1, u_r = sq x_r
    // (the same products the stored form would hold); column i is rewritten
    // in that form only after the update, so no barrier precedes it.
    const bool merged = m - i <= kZRows;
    const float* uc = M + (size_t)i * ld;
    if (merged) {
      switch (row_slices(m - i)) {
        case 1: left_pass<1>(M, ld, m, n, i, tauq, sq, zs, lane, wid, nw); break;
        case 2: left_pass<2>(M, ld, m, n, i, tauq, sq, zs, lane, wid, nw); break;
        case 4: left_pass<4>(M, ld, m, n, i, tauq, sq, zs, lane, wid, nw); break;
        default: left_pass<8>(M, ld, m, n, i, tauq, sq, zs, lane, wid, nw); break;
      }
    } else if (tauq != 0.f) {
      for (int c = i + 1 + wid; c < n; c += nw) {
        float* col = M + (size_t)c * ld;
        float w = 0.f;
        for (int r = i + lane; r < m; r += 32) w += (r == i ? 1.f : uc[r] * sq) * col[r];
        w = warp_sum(w) * tauq;
        for (int r = i + lane; r < m; r += 32) col[r] -= w * (r == i ? 1.f : uc[r] * sq);
      }
    }
    __syncthreads();
    BMARK(tr ? i : 999, 2, global_ns());
    // column i in reflector form (no later step of this problem reads it);
    // warp 0 meanwhile forms the right reflector from row i (disjoint
    // entries), and every thread adds the warps' partial products of its rows
    if (t == 0) M[i + (size_t)i * ld] = 1.f;
    for (int r = i + 1 + t; r < m; r += blockDim.x) M[r + (size_t)i * ld] *= sq;
    if (merged)
      for (int rr = 1 + t; rr < m - i; rr += blockDim.x) {
        float z = 0.f;
        for (int w = 0; w < nw; w++) z += zs[w * kZRows + rr];
        zsum[rr] = z;
      }
    if (wid == 0) {
      const float y0 = M[i + (size_t)(i + 1) * ld];
      FF r2{0.f, 0.f};
      for (int c = i + 2 + lane; c < n; c += 32) r2 = ff_add_sq(r2, M[i + (size_t)c * ld]);
      r2 = warp_sum_ff(r2);
      float beta, taup, sp;
      if (i < n - 2) {
        householder_ff(y0, r2, &beta, &taup, &sp);
      } else {  // one element left: no reflection (bidiag.c:125-129)
        beta = y0;
        taup = 0.f;
        sp = 0.f;
      }
      if (lane == 0) {
        e[i] = beta;
        tp[i] = taup;
        sh[2] = taup;
        sh[3] = sp;
      }
      for (int c = i + 1 + lane; c < n; c += 32) {
        const float v = (c == i + 1) ? ((taup != 0.f) ? 1.f : 0.f) : M[i + (size_t)c * ld] * sp;
        M[i + (size_t)c * ld] = v;
        vrow[c] = v;
      }
    }
    __syncthreads();
    BMARK(tr ? i : 999, 3, global_ns());
    const float taup = sh[2], sp = sh[3];
    // ---- right update of rows > i (right_dotprods + right_update_mat):
    // two threads per row (alternate columns) while the rows fit, so every
    // thread works (more threads per row measured slower: shuffles and
    // shared-memory bank conflicts)
    if (taup != 0.f) {
      if (2 * (m - i - 1) <= (int)blockDim.x) {
        const int r = i + 1 + (t >> 1), h = t & 1;
        const bool act = r < m;
        float z = 0.f;
        if (merged) {
          if (act) z = M[r + (size_t)(i + 1) * ld] + sp * zsum[r - i];
          __syncwarp();  // both threads of the row read a_{r,i+1} before it changes
        } else {
          if (act)
            for (int c = i + 1 + h; c < n; c += 2) z += M[r + (size_t)c * ld] * vrow[c];
          z += __shfl_xor_sync(0xffffffffu, z, 1);
        }
        z *= taup;
        if (act)
          for (int c = i + 1 + h; c < n; c += 2) M[r + (size_t)c * ld] -= z * vrow[c];
      } else {
        for (int r = i + 1 + t; r < m; r += blockDim.x) {
          float z = 0.f;
          if (merged) {
            z = M[r + (size_t)(i + 1) * ld] + sp * zsum[r - i];
          } else {
            for (int c = i + 1; c < n; c++) z += M[r + (size_t)c * ld] * vrow[c];
          }
          z *= taup;
          for (int c = i + 1; c < n; c++) M[r + (size_t)c * ld] -= z * vrow[c];
        }
      }
    }
    __syncthreads();
    BMARK(tr ? i : 999, 4, global_ns());
  }
}

__global__ void __launch_bounds__(kBatchBidiagThreads) batch_bidiag_kernel(const BatchTask* __restrict__ tasks,
                                                                     const int* __restrict__ order, int ntask,
                                                                     int* counter, const float* __restrict__ A,
                                                                     float* W, float* d, float* e, float* tq,
                                                                     float* tp, int smem_floats, int maxn) {
  extern __shared__ __align__(16) float sm[];
  __shared__ int s_task;
  __shared__ float red[4];  // reflector scalars handed from warp 0 to the CTA
  __shared__ unsigned s_amax;
  float* vrow = sm;                                   // maxn
  float* zs = sm + ((maxn + 3) & ~3);  // right products: warps x 256 partials + 256 totals
  float* Ms = zs + ((blockDim.x >> 5) + 1) * 32 * kColRegs;  // problem copy when it fits
#ifdef DDCSVD_PHASE_TRACE
  int pcount = 0;
#endif
  while (true) {
    if (threadIdx.x == 0) s_task = atomicAdd(counter, 1);
    __syncthreads();
    const int q = s_task;
    __syncthreads();
    if (q >= ntask) break;
    const BatchTask T = tasks[order[q]];
    const int m = T.m, n = T.n, ld = m;
#ifdef DDCSVD_PHASE_TRACE
    const int prow = 64 + pcount;
    const bool first = pcount == 0;
    BMARK(prow, 0, global_ns());
    BMARK(prow, 2, (unsigned long long)m);
    BMARK(prow, 3, (unsigned long long)n);
#else
    const bool first = false;
#endif
    const bool fits = (long long)m * n <= smem_floats;
    // a problem beyond the shared memory: columns [0, k0) run in global memory
    // until the trailing block fits (k0 = n: none fits)
    int k0 = 0;
    if (!fits)
      while (k0 < n && (long long)(m - k0) * (n - k0) > smem_floats) k0++;
    float* Wg = W + T.offW;
    float* M = fits ? Ms : Wg;
    // load the (oriented) problem; max|a| for the range scaling of the norms
    const float* src = A + T.offA;
    if (threadIdx.x == 0) s_amax = 0u;
    float amax = 0.f;
    for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) {
      const int r = idx % m, c = idx / m;
      const float v = T.trans ? src[c + (size_t)r * n] : src[idx];
      M[r + (size_t)c * ld] = v;
      amax = fmaxf(amax, fabsf(v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && amax > 0.f) atomicMax(&s_amax, __float_as_uint(amax));
    __syncthreads();
    const float sc = range_scale(s_amax);
    if (sc != 1.f)
      for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) M[(idx % m) + (size_t)(idx / m) * ld] *= sc;
    __syncthreads();
    if (fits || k0 >= n) {
      cta_bidiag(M, ld, m, n, d + T.offD, e + T.offD, tq + T.offD, tp + T.offD, vrow, zs, red, n, first);
    } else {
      // the first k0 columns in global memory, then the (m - k0) x (n - k0)
      // trailing block (the only part later columns touch) in shared memory
      cta_bidiag(M, ld, m, n, d + T.offD, e + T.offD, tq + T.offD, tp + T.offD, vrow, zs, red, k0);
      __syncthreads();
      const int mt = m - k0, nt = n - k0;
      for (int idx = threadIdx.x; idx < mt * nt; idx += blockDim.x)
        Ms[idx] = Wg[(k0 + idx % mt) + (size_t)(k0 + idx / mt) * ld];
      __syncthreads();
      cta_bidiag(Ms, mt, mt, nt, d + T.offD + k0, e + T.offD + k0, tq + T.offD + k0, tp + T.offD + k0, vrow, zs,
                 red, nt);
      __syncthreads();
      for (int idx = threadIdx.x; idx < mt * nt; idx += blockDim.x)
        Wg[(k0 + idx % mt) + (size_t)(k0 + idx / mt) * ld] = Ms[idx];
    }
    __syncthreads();
    if (sc != 1.f) {
      const float inv = 1.f / sc;
      for (int k = threadIdx.x; k < n; k += blockDim.x) {
        d[T.offD + k] *= inv;
        if (k < n - 1) e[T.offD + k] *= inv;
      }
    }
    if (fits)
      for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) Wg[idx] = M[idx];
    __syncthreads();
#ifdef DDCSVD_PHASE_TRACE
    BMARK(prow, 1, global_ns());
    pcount++;
#endif
  }
}

// Applies reflectors j = jhi-1 ... 0 to kCW columns held in registers (lane
// owns rows lane + 32 k, k < KR).  Reflector j is the vector v(r) = vec(j, r)
// for rows r >= j + shift (unit leading entry stored), zero above.  KR is the
// problem's row count in 32-row slices (1, 2, 4 or 8), so small problems do
// not multiply zeros.  The kCW dot products of a reflector are summed over
// the warp by a reduce-scatter (4 + 2 + 1 shuffles leave each lane a partial
// of one column over 8 lanes, 2 more complete it) and a gather of the 8
// sums (17 shuffles instead of 5 per column).
constexpr int kCW = 8;  // columns per warp at a time
template <int KR, typename VecFn>
__device__ __forceinline__ void apply_reflectors_regs(float (&c)[kCW][KR], int rows, int jhi, int shift,
                                                      const float* __restrict__ tau, VecFn vec, int lane) {
  const bool b16 = lane & 16, b8 = lane & 8, b4 = lane & 4;
  for (int j = jhi - 1; j >= 0; j--) {
    const float t = tau[j];
    if (t == 0.f) continue;
    float u[KR];
#pragma unroll
    for (int k = 0; k < KR; k++) {
      const int r = lane + 32 * k;
      u[k] = (r >= j + shift && r < rows) ? vec(j, r) : 0.f;
    }
    float d[kCW];
#pragma unroll
    for (int q = 0; q < kCW; q++) {
      float a = 0.f;
#pragma unroll
      for (int k = 0; k < KR; k++) a += u[k] * c[q][k];
      d[q] = a;
    }
    float e4[4], e2[2];
#pragma unroll
    for (int q = 0; q < 4; q++)
      e4[q] = (b16 ? d[q + 4] : d[q]) + __shfl_xor_sync(0xffffffffu, b16 ? d[q] : d[q + 4], 16);
#pragma unroll
    for (int q = 0; q < 2; q++)
      e2[q] = (b8 ? e4[q + 2] : e4[q]) + __shfl_xor_sync(0xffffffffu, b8 ? e4[q] : e4[q + 2], 8);
    float g = (b4 ? e2[1] : e2[0]) + __shfl_xor_sync(0xffffffffu, b4 ? e2[0] : e2[1], 4);
    g += __shfl_xor_sync(0xffffffffu, g, 2);
    g += __shfl_xor_sync(0xffffffffu, g, 1);
    // lane l now holds the sum of column 4 b16 + 2 b8 + b4
#pragma unroll
    for (int q = 0; q < kCW; q++) {
      const float f = t * __shfl_sync(0xffffffffu, g, ((q >> 2) & 1) * 16 + ((q >> 1) & 1) * 8 + (q & 1) * 4);
#pragma unroll
      for (int k = 0; k < KR; k++) c[q][k] -= f * u[k];
    }
  }
}

// Left side of one problem up to 256 rows: U_core = Q [Y; 0], kCW columns per
// warp at a time in registers, left reflectors n-1 .. 0 (column j of R).
template <int KR>
__device__ void bx_left(float* Uc, int m, int n, const float* R, const float* tauq, int lane, int wid, int nw) {
  for (int c0 = wid * kCW; c0 < n; c0 += nw * kCW) {
    float c[kCW][KR];
#pragma unroll
    for (int qq = 0; qq < kCW; qq++)
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = lane + 32 * k, col = c0 + qq;
        c[qq][k] = (col < n && r < n) ? Uc[r + (size_t)col * m] : 0.f;
      }
    apply_reflectors_regs<KR>(c, m, n, 0, tauq, [&](int j, int r) { return R[r + (size_t)j * m]; }, lane);
#pragma unroll
    for (int qq = 0; qq < kCW; qq++)
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = lane + 32 * k, col = c0 + qq;
        if (col < n && r < m) Uc[r + (size_t)col * m] = c[qq][k];
      }
  }
}

// Right side: V_core = P X, right reflectors n-3 .. 0 (row j of R from column j+1).
template <int KR>
__device__ void bx_right(float* Vc, int m, int n, const float* R, const float* taup, int lane, int wid, int nw) {
  for (int c0 = wid * kCW; c0 < n; c0 += nw * kCW) {
    float c[kCW][KR];
#pragma unroll
    for (int qq = 0; qq < kCW; qq++)
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = lane + 32 * k, col = c0 + qq;
        c[qq][k] = (col < n && r < n) ? Vc[r + (size_t)col * n] : 0.f;
      }
    apply_reflectors_regs<KR>(c, n, n - 2, 1, taup, [&](int j, int k) { return R[j + (size_t)k * m]; }, lane);
#pragma unroll
    for (int qq = 0; qq < kCW; qq++)
#pragma unroll
      for (int k = 0; k < KR; k++) {
        const int r = lane + 32 * k, col = c0 + qq;
        if (col < n && r < n) Vc[r + (size_t)col * n] = c[qq][k];
      }
  }
}

// U_core = Q [Y; 0], V_core = P X for one problem per CTA (multU / multV).
// Persistent CTAs take problems largest first from an atomic counter over the
// size-sorted order (a static round robin left the largest problems to the
// last wave).  Problems up to 256 rows keep kCW columns per warp in
// registers, sized to the problem's rows, and read the reflectors from
// shared memory (or L1): one warp-wide reduction per reflector for kCW
// columns at once.  Larger problems use the plain column loop (one column
// per warp, in global memory).
__global__ void __launch_bounds__(kBatchThreads) batch_backxform_kernel(const BatchTask* __restrict__ tasks,
                                                                        const int* __restrict__ order, int ntask,
                                                                        int* counter, const float* __restrict__ W,
                                                                        const float* __restrict__ tq,
                                                                        const float* __restrict__ tp, float* U,
                                                                        float* V, int smem_floats) {
  extern __shared__ __align__(16) float sm[];
  __shared__ int s_task;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  while (true) {
    if (threadIdx.x == 0) s_task = atomicAdd(counter, 1);
    __syncthreads();
    const int qi = s_task;
    if (qi >= ntask) break;
    const BatchTask T = tasks[order[qi]];
    const int m = T.m, n = T.n;
    const bool fits = (long long)m * n <= smem_floats;
    const float* Wg = W + T.offW;
    if (fits)
      for (int idx = threadIdx.x; idx < m * n; idx += blockDim.x) sm[idx] = Wg[idx];
    const float* R = fits ? sm : Wg;
    // core U / V of a transposed problem are the caller's V / U
    float* Uc = (T.trans ? V : U) + T.offU;
    float* Vc = (T.trans ? U : V) + T.offV;
    __syncthreads();
    const float* tauq = tq + T.offD;
    const float* taup = tp + T.offD;
    if (m <= 256) {
      switch (row_slices(m)) {
        case 1: bx_left<1>(Uc, m, n, R, tauq, lane, wid, nw); break;
        case 2: bx_left<2>(Uc, m, n, R, tauq, lane, wid, nw); break;
        case 4: bx_left<4>(Uc, m, n, R, tauq, lane, wid, nw); break;
        default: bx_left<8>(Uc, m, n, R, tauq, lane, wid, nw); break;
      }
      switch (row_slices(n)) {
        case 1: bx_right<1>(Vc, m, n, R, taup, lane, wid, nw); break;
        case 2: bx_right<2>(Vc, m, n, R, taup, lane, wid, nw); break;
        case 4: bx_right<4>(Vc, m, n, R, taup, lane, wid, nw); break;
        default: bx_right<8>(Vc, m, n, R, taup, lane, wid, nw); break;
      }
    } else {
      // rows n..m-1 of [Y; 0]
      for (int idx = threadIdx.x; idx < (m - n) * n; idx += blockDim.x) {
        const int r = n + idx % (m - n), c = idx / (m - n);
        Uc[r + (size_t)c * m] = 0.f;
      }
      __syncthreads();
      for (int c = wid; c < n; c += nw) {
        float* col = Uc + (size_t)c * m;
        for (int j = n - 1; j >= 0; j--) {
          const float t = tauq[j];
          if (t == 0.f) continue;
          const float* u = R + (size_t)j * m;  // unit stored at u[j]
          float s = 0.f;
          for (int r = j + lane; r < m; r += 32) s += u[r] * col[r];
          s = warp_sum(s) * t;
          for (int r = j + lane; r < m; r += 32) col[r] -= s * u[r];
          __syncwarp();
        }
        float* vc = Vc + (size_t)c * n;
        for (int j = n - 3; j >= 0; j--) {
          const float t = taup[j];
          if (t == 0.f) continue;
          float s = 0.f;  // right reflector j: row j of R from column j+1 (unit stored)
          for (int k = j + 1 + lane; k < n; k += 32) s += R[j + (size_t)k * m] * vc[k];
          s = warp_sum(s) * t;
          for (int k = j + 1 + lane; k < n; k += 32) vc[k] -= s * R[j + (size_t)k * m];
          __syncwarp();
        }
      }
    }
    __syncthreads();
  }
}

__global__ void batch_sigma_out_kernel(const BatchTask* __restrict__ tasks, int ntask, const double* sig,
                                       float* S) {
  for (int q = blockIdx.x; q < ntask; q += gridDim.x) {
    const BatchTask T = tasks[q];
    for (int i = threadIdx.x; i < T.n; i += blockDim.x) S[T.offS + i] = (float)sig[T.offD + i];
  }
}

}  // namespace ddcsvd

using namespace ddcsvd;

extern "C" int ddcsvd_svd_batched_f32_device(ddcsvd_handle_t h, int batch, const int* m, const int* n,
                                             const float* dA, const long long* offA, float* dSigma,
                                             const long long* offS, float* dU, const long long* offU,
                                             float* dV, const long long* offV) {
  if (!h || batch <= 0 || !m || !n || !dA || !offA || !dSigma || !offS || !dU || !offU || !dV || !offV)
    return DDCSVD_ERR_ARG;
  for (int b = 0; b < batch; b++)
    if (m[b] <= 0 || n[b] <= 0) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  // ---- task table (oriented so that m >= n)
  std::vector<BatchTask> tasks(batch);
  std::vector<int> gn(batch);
  std::vector<GroupOut> gout(batch);
  long long offW = 0, offD = 0;
  int maxn = 0;
  long long maxmn = 0;
  for (int b = 0; b < batch; b++) {
    BatchTask& T = tasks[b];
    T.trans = m[b] < n[b];
    T.m = std::max(m[b], n[b]);
    T.n = std::min(m[b], n[b]);
    T.pad = 0;
    T.offW = offW;
    T.offD = offD;
    T.offA = offA[b];
    T.offS = offS[b];
    // core U (m x n) is the caller's U, or V when transposed; same for core V
    T.offU = T.trans ? offV[b] : offU[b];
    T.offV = T.trans ? offU[b] : offV[b];
    offW += (long long)T.m * T.n;
    offD += T.n;
    maxn = std::max(maxn, T.n);
    maxmn = std::max(maxmn, (long long)T.m * T.n);
    gn[b] = T.n;
    float* Ucore = T.trans ? dV : dU;
    float* Vcore = T.trans ? dU : dV;
    gout[b] = GroupOut{Vcore + T.offV, T.n, Ucore + T.offU, T.m};
  }
  const int Ntot = (int)offD;
  std::vector<int> order(batch);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (long long)tasks[x].m * tasks[x].n > (long long)tasks[y].m * tasks[y].n;
  });
  const PrepBounds PB = prep_bounds(gn);
  // ---- workspace
  auto layout = [&](Arena& a, float** W, float** d, float** e, float** tq, float** tp, BatchTask** dt, int** dord,
                    int** counter, char** blob, double** sig_slot, double** sig) {
    *W = a.take<float>(offW + 64);
    *d = a.take<float>(Ntot + 8);
    *e = a.take<float>(Ntot + 8);
    *tq = a.take<float>(Ntot + 8);
    *tp = a.take<float>(Ntot + 8);
    *dt = a.take<BatchTask>(batch);
    *dord = a.take<int>(batch);
    *counter = a.take<int>(8);
    *blob = a.take<char>(PB.blob_bytes);
    *sig_slot = a.take<double>(Ntot + 8);
    *sig = a.take<double>(Ntot + 8);
  };
  float *W, *d, *e, *tq, *tp;
  BatchTask* dt;
  int *dord, *counter;
  char* blob;
  double *sig_slot, *sig;
  size_t need;
  {
    Arena a;
    layout(a, &W, &d, &e, &tq, &tp, &dt, &dord, &counter, &blob, &sig_slot, &sig);
    Arena b = a, c = a;
    DDC_TRY(dc_sigma(h, Ntot, nullptr, nullptr, nullptr, nullptr, nullptr, b, true));
    DDC_TRY(bd_vectors(h, Ntot, PB.store, nullptr, nullptr, nullptr, nullptr, nullptr, c, true));
    need = std::max(b.off, c.off);
  }
  DDC_TRY(ensure_workspace(h, need + 4096));
  Arena a;
  a.plan = false;
  a.base = (char*)h->ws;
  layout(a, &W, &d, &e, &tq, &tp, &dt, &dord, &counter, &blob, &sig_slot, &sig);
  // ---- pinned staging: tasks + order, then (after stage 1) the bidiagonal and the prep blob
  const size_t tb = (size_t)round_up(sizeof(BatchTask) * batch + sizeof(int) * batch + 64, 256);
  const size_t rb = (size_t)round_up(sizeof(float) * 2 * (Ntot + 8), 256);
  const size_t ab = (size_t)round_up(sizeof(double) * 2 * (Ntot + 8), 256);
  DDC_TRY(ensure_pinned(h, tb + rb + ab + PB.blob_bytes));
  char* pin = (char*)h->pinned;
  memcpy(pin, tasks.data(), sizeof(BatchTask) * batch);
  memcpy(pin + sizeof(BatchTask) * batch, order.data(), sizeof(int) * batch);
  DDC_TRY(reset_status(h));
  h->kused = 0;
  DDC_CUDA_TRY(cudaMemcpyAsync(dt, pin, sizeof(BatchTask) * batch, cudaMemcpyHostToDevice, h->stream));
  DDC_CUDA_TRY(cudaMemcpyAsync(dord, pin + sizeof(BatchTask) * batch, sizeof(int) * batch, cudaMemcpyHostToDevice,
                               h->stream));
  DDC_CUDA_TRY(cudaMemsetAsync(counter, 0, 2 * sizeof(int), h->stream));  // stage 1 and stage 5 work counters
  // ---- stage 1: persistent CTAs over the size-sorted work list
  // stage 1 keeps a problem in shared memory when it fits the SM's opt-in
  // maximum (up to ~56K entries: all but the largest 256 x 2xx problems);
  // stage 5 reads its reflectors from up to 24K entries of shared memory
  const int smem_floats = 24 * 1024;
  int max_optin = 0;
  DDC_CUDA_TRY(cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
  const int bthreads = (h->tune[TK_BATCH_THREADS] == 256) ? 256 : kBatchBidiagThreads;
  const int vrow_floats = (int)((maxn + 3) & ~3) + (bthreads / 32 + 1) * 32 * kColRegs;
  const int bidiag_floats = h->tune[TK_BATCH_SMEM_FULL]
                                ? std::max(1024, (max_optin - 2048) / (int)sizeof(float) - vrow_floats)
                                : smem_floats;
  const size_t smem = sizeof(float) * ((size_t)vrow_floats + bidiag_floats);
  DDC_CUDA_TRY(cudaFuncSetAttribute(batch_bidiag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 1;
  DDC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_bidiag_kernel, bthreads, smem));
  const int grid1 = std::max(1, std::min(batch, h->num_sms * std::max(occ, 1)));
  ktimer_begin(h, KC_BIDIAG);
  batch_bidiag_kernel<<<grid1, bthreads, smem, h->stream>>>(dt, dord, batch, counter, dA, W, d, e, tq,
                                                                       tp, bidiag_floats, maxn);
  ktimer_end(h);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  // ---- bidiagonal read-back and preparation (one forest, one group per problem)
  float* hd = (float*)(pin + tb);
  float* he = hd + Ntot + 8;
  DDC_CUDA_TRY(cudaMemcpyAsync(hd, d, sizeof(float) * Ntot, cudaMemcpyDeviceToHost, h->stream));
  DDC_CUDA_TRY(cudaMemcpyAsync(he, e, sizeof(float) * Ntot, cudaMemcpyDeviceToHost, h->stream));
  DDC_CUDA_TRY(cudaMemcpyAsync(h->h_status, h->d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->stream));
  // while stage 1 runs: the D&C forest and vector layout for one block per
  // problem (a split inside a problem is rare; prep_build lays out anew then)
  Prep P;
  {
    std::vector<int> starts0;
    starts0.reserve(batch + 1);
    int off = 0;
    for (int b = 0; b < batch; b++) {
      if (gn[b] > 0) starts0.push_back(off);
      off += gn[b];
    }
    starts0.push_back(off);
    DDC_TRY(prep_layout(h, gn, gout, starts0, pin + tb + rb + ab, blob, &P));
  }
  DDC_CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (h->h_status->code != 0) {  // a stage-1 failure ends the call before stages 2-5
    set_last_error("batched bidiagonalisation: device status %d (detail %d)", h->h_status->code,
                   h->h_status->detail);
    return h->h_status->code;
  }
  double* a64 = (double*)(pin + tb + rb);
  double* b64 = a64 + Ntot + 8;
  for (int b = 0; b < batch; b++) {
    const long long o = tasks[b].offD;
    const int nb = tasks[b].n;
    for (int i = 0; i < nb; i++) {
      a64[o + i] = hd[o + i];
      b64[o + i] = (i < nb - 1) ? (double)he[o + i] : 0.0;
    }
  }
  DDC_TRY(prep_build(h, gn, gout, a64, b64, FLT_EPSILON, false, pin + tb + rb + ab, blob, &P));
  // ---- stages 2-4
  {
    Arena b = a;
    DDC_TRY(dc_sigma(h, Ntot, P.b1, P.b2, sig_slot, &P.H, P.dints, b, false));
  }
  {
    Arena c = a;
    DDC_TRY(bd_vectors(h, Ntot, P.store, P.b1, P.b2, sig_slot, &P.L, sig, c, false));
  }
  // ---- stage 5 and sigma
  const size_t smem5 = sizeof(float) * (size_t)std::min<long long>(maxmn, smem_floats);
  DDC_CUDA_TRY(cudaFuncSetAttribute(batch_backxform_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)std::max<size_t>(smem5, 16)));
  ktimer_begin(h, KC_BACKXFORM);
  int occ5 = 1;
  DDC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ5, batch_backxform_kernel, kBatchThreads,
                                                            std::max<size_t>(smem5, 16)));
  batch_backxform_kernel<<<std::min(batch, h->num_sms * std::max(occ5, 1)), kBatchThreads, smem5, h->stream>>>(
      dt, dord, batch, counter + 1, W, tq, tp, dU, dV, smem_floats);
  count_launch();
  ktimer_end(h);
  batch_sigma_out_kernel<<<std::min(batch, 1024), 128, 0, h->stream>>>(dt, batch, sig, dSigma);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  const int rc = check_status(h, "svd_batched");
  if (h->timing && rc == DDCSVD_OK) ktimer_collect(h);
  return rc;
}

#ifdef DDCSVD_PHASE_TRACE
extern "C" int ddcsvd_batch_trace_read(unsigned long long* out) {
  return (int)cudaMemcpyFromSymbol(out, ddcsvd::g_batch_trace, sizeof(ddcsvd::g_batch_trace));
}
#endif
