// tail.cu -- the last columns of the blocked bidiagonalisation on one
// thread-block cluster.
//
// Once the trailing block W[k0:m, k0:n] of the panel factorisation is small
// enough to live in the distributed shared memory of one cluster (C CTAs,
// C = 16 where the GPU can co-schedule that many, else 8), the remaining
// columns no longer pay the grid-wide costs of the panel kernel (two grid
// barriers and two reductions over 152 partial records per column, ~9 us at
// any size).  Here CTA k holds columns k, k + C, k + 2C, ... of the trailing
// block (cyclic, so the work stays even while columns retire), all rows, in
// its shared memory and the algorithm is the unblocked one of
// the reference (bidiag_par.c:310-397, left_update_mat.cl / right_update_mat.cl):
// per column a left reflector and its rank-1 update, then a right reflector
// and its rank-1 update, exchanged through distributed shared memory with
// four hardware cluster barriers.  Reflector conventions, FP32 compensated
// norms and the LAPACK-form storage are those of the panel kernel, so the
// back-transformation reads the result unchanged.
//
// The unblocked form rewrites the trailing block every column at the shared-
// memory bandwidth of C SMs, so it only beats the 152-SM panel kernel once
// the block is small: measured on 4096^2 / 2048^2 / 1024^2 SVDs, handing over
// the last 512 columns is best (77.4 -> 75.9, 30.2 -> 28.8, 14.8 -> 13.3 ms;
// the last 384 or 640 columns slightly worse, every column that fits -- ~900
// at 4096^2 -- slower than none).  A 512 x 256 problem runs here entirely
// (4.5 -> 3.7 ms).
#include <cooperative_groups.h>

#include "internal.hpp"

namespace cg = cooperative_groups;

namespace ddcsvd {

constexpr int kTailThreads = 512;

// phase marks (trace builds): CTA 0, every 8th column, one row per column
#ifdef DDCSVD_PHASE_TRACE
__device__ unsigned long long g_tail_trace[128 * 16];
#define TMARK(slot)                                                                  \
  do {                                                                               \
    if (rank == 0 && threadIdx.x == 0 && (i & 7) == 0 && (i >> 3) < 128)             \
      g_tail_trace[(i >> 3) * 16 + (slot)] = global_ns();                            \
  } while (0)
#else
#define TMARK(slot) \
  do {              \
  } while (0)
#endif

struct TailParams {
  int mt, nt;     // trailing block: rows, columns (mt >= nt)
  int ncb;        // columns per CTA (at most)
  float* W;       // trailing block (its row 0 / column 0 = the first tail column)
  int ldw;
  float *d, *e, *tauq, *taup;  // offset to the first tail column
};

// Shared-memory layout (floats, every section 16-byte aligned): A [mt x ncb]
// (column-major, ld mt), u, xp, xs, x [mt each], red [32 FF], scal [8],
// nrm [1 FF].
__host__ __device__ inline size_t tail_vec_floats(int mt) { return (size_t)((mt + 4 + 3) & ~3); }
__host__ __device__ inline size_t tail_smem_floats(int mt, int ncb) {
  return (((size_t)mt * ncb + 3) & ~(size_t)3) + 4 * tail_vec_floats(mt) + 64 + 8 + 4;
}

// CTA-wide compensated sum (fixed order: warp trees, then warps in order).
__device__ __forceinline__ FF tail_sum_ff(FF v, FF* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum_ff(v);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    FF s = lane < nw ? red[lane] : FF{0.f, 0.f};
    s = warp_sum_ff(s);
    if (lane == 0) red[0] = s;
  }
  __syncthreads();
  return red[0];
}

__global__ void __launch_bounds__(kTailThreads, 1) bidiag_tail_kernel(TailParams p) {
  extern __shared__ __align__(16) float sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5, nt_ = blockDim.x;
  const int mt = p.mt, ncols = p.nt, ncb = p.ncb;
  // own columns: c = rank + l * C, l < nown (local index l)
  const int nown = rank < ncols ? (ncols - rank + C - 1) / C : 0;
  // first local index whose column is >= c
  auto lfirst = [&](int c) { return c <= rank ? 0 : (c - rank + C - 1) / C; };
  float* A = sm;
  float* u = A + (((size_t)mt * ncb + 3) & ~(size_t)3);
  float* xp = u + tail_vec_floats(mt);
  float* xs = xp + tail_vec_floats(mt);
  float* x = xs + tail_vec_floats(mt);
  FF* red = reinterpret_cast<FF*>(x + tail_vec_floats(mt));
  float* scal = reinterpret_cast<float*>(red + 32);
  FF* nrm = reinterpret_cast<FF*>(scal + 8);

  // own columns into shared memory
  for (int l = 0; l < nown; l++)
    for (int r = t; r < mt; r += nt_) A[r + (size_t)l * mt] = p.W[r + (size_t)(rank + l * C) * p.ldw];
  __syncthreads();
  cluster.sync();

  for (int i = 0; i < ncols; i++) {
    const int own_i = i % C;  // rank owning column i (its local index i / C)
    TMARK(0);
    // ---- A: left reflector from column i (its owner)
    if (rank == own_i) {
      float* col = A + (size_t)(i / C) * mt;
      FF s2{0.f, 0.f};
      for (int r = i + 1 + t; r < mt; r += nt_) s2 = ff_add_sq(s2, col[r]);
      s2 = tail_sum_ff(s2, red);
      float alpha, tq, sq;
      householder_ff(col[i], s2, &alpha, &tq, &sq);
      __syncthreads();  // col[i] read by every thread before it is overwritten
      for (int r = i + t; r < mt; r += nt_) col[r] = (r == i) ? 1.f : col[r] * sq;
      if (t == 0) {
        p.d[i] = alpha;
        p.tauq[i] = tq;
        scal[0] = tq;
      }
    }
    TMARK(1);
    cluster.sync();  // #1: u and tau_q published
    TMARK(2);
    // ---- B: left update of the own columns > i, partial norm of row i
    {
      const float* ucol = cluster.map_shared_rank(A + (size_t)(i / C) * mt, own_i);
      const float tq = *cluster.map_shared_rank(scal, own_i);
      for (int r = i + t; r < mt; r += nt_) u[r] = ucol[r];
      __syncthreads();
      if (tq != 0.f) {
        for (int l = lfirst(i + 1) + wid; l < nown; l += nw) {  // warp per column
          float* col = A + (size_t)l * mt;
          float y = 0.f;
          for (int r = i + lane; r < mt; r += 32) y += u[r] * col[r];
          y = warp_sum(y) * tq;
          for (int r = i + lane; r < mt; r += 32) col[r] -= y * u[r];
        }
      }
      __syncthreads();
      FF s{0.f, 0.f};
      for (int l = lfirst(i + 2) + t; l < nown; l += nt_) s = ff_add_sq(s, A[i + (size_t)l * mt]);
      s = tail_sum_ff(s, red);
      if (t == 0) {
        *nrm = s;
        // the row's first element, published before its owner overwrites it in C
        if (i + 1 < ncols && (i + 1) % C == rank) scal[3] = A[i + (size_t)((i + 1) / C) * mt];
      }
    }
    if (i == ncols - 1) break;  // last column: no right reflector
    TMARK(3);
    cluster.sync();  // #2: row-norm partials published
    TMARK(4);
    // ---- C: right reflector from row i (every CTA forms it), partial x
    float tp;
    {
      if (t < 32) {
        // the C partial norms fetched by lanes 0..C-1 at once, added by one shuffle tree
        FF v = t < C ? *cluster.map_shared_rank(nrm, t) : FF{0.f, 0.f};
        const FF tot = warp_sum_ff(v);
        const float x0 = *cluster.map_shared_rank(scal + 3, (i + 1) % C);
        float beta, tpv, sp;
        if (i < ncols - 2) {
          householder_ff(x0, tot, &beta, &tpv, &sp);
        } else {  // one element left: no reflection (bidiag.c:125-129)
          beta = x0;
          tpv = 0.f;
          sp = 0.f;
        }
        if (t == 0) {
          if (rank == 0) {
            p.e[i] = beta;
            p.taup[i] = tpv;
          }
          scal[1] = tpv;
          scal[2] = sp;
        }
      }
      __syncthreads();
      TMARK(5);
      tp = scal[1];
      const float sp = scal[2];
      const int lf = lfirst(i + 1);
      for (int l = lf + t; l < nown; l += nt_) {
        float* a = A + i + (size_t)l * mt;
        *a = (rank + l * C == i + 1) ? (tp != 0.f ? 1.f : 0.f) : *a * sp;
      }
      __syncthreads();
      for (int r = i + 1 + t; r < mt; r += nt_) {
        float s = 0.f;
        for (int l = lf; l < nown; l++) s += A[r + (size_t)l * mt] * A[i + (size_t)l * mt];
        xp[r] = s;
      }
    }
    TMARK(6);
    cluster.sync();  // #3: partial x published
    TMARK(7);
    // ---- D: x = sum of the C partials (reduce-scatter, all-gather), right update
    {
      const int len = ceil_div(mt - i - 1, C);
      const int s0 = i + 1 + rank * len, s1 = min(mt, s0 + len);
      for (int r = s0 + t; r < s1; r += nt_) {
        float s = 0.f;
        for (int k = 0; k < C; k++) s += cluster.map_shared_rank(xp, k)[r];
        xs[r] = s;
      }
      TMARK(8);
      cluster.sync();  // #4: slices of x published
      TMARK(9);
      for (int r = i + 1 + t; r < mt; r += nt_) x[r] = cluster.map_shared_rank(xs, (r - i - 1) / len)[r];
      __syncthreads();
      if (tp != 0.f) {
        const int lf = lfirst(i + 1);
        for (int r = i + 1 + t; r < mt; r += nt_) {
          const float f = tp * x[r];
          for (int l = lf; l < nown; l++) A[r + (size_t)l * mt] -= f * A[i + (size_t)l * mt];
        }
      }
      __syncthreads();
      TMARK(10);
    }
  }
  // reflectors and the bidiagonal's neighbourhood back to the working matrix
  cluster.sync();
  for (int l = 0; l < nown; l++)
    for (int r = t; r < mt; r += nt_) p.W[r + (size_t)(rank + l * C) * p.ldw] = A[r + (size_t)l * mt];
}

// Cluster size the device can co-schedule (16, else 8, else 0), cached.
static int tail_cluster_size(ddcsvd_context* ctx) {
  if (ctx->tail_cluster >= 0) return ctx->tail_cluster;
  int best = 0;
  if (cudaFuncSetAttribute((const void*)bidiag_tail_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
      cudaSuccess) {
    const int smem = (int)(ctx->smem_optin > 1024 ? ctx->smem_optin - 1024 : ctx->smem_optin);
    cudaFuncSetAttribute((const void*)bidiag_tail_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    for (int c : {16, 8}) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(kTailThreads);
      cfg.dynamicSmemBytes = smem;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = c;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)bidiag_tail_kernel, &cfg) == cudaSuccess &&
          nclusters >= 1) {
        best = c;
        break;
      }
    }
  }
  cudaGetLastError();  // a refused attribute or query only means no cluster tail
  ctx->tail_cluster = best;
  return best;
}

int bidiag_tail_columns(ddcsvd_context* ctx, int m, int n, int k0) {
  const int cap = ctx->tune[TK_PANEL_TAIL];
  const int mt = m - k0, nt = n - k0;
  if (cap <= 0 || nt > cap || nt <= 0 || mt < nt) return 0;
  const int C = tail_cluster_size(ctx);
  if (C == 0) return 0;
  const int ncb = ceil_div(nt, C);
  const size_t bytes = tail_smem_floats(mt, ncb) * sizeof(float);
  return (bytes + 1024 <= ctx->smem_optin) ? nt : 0;
}

int bidiag_tail(ddcsvd_context* ctx, int m, int n, int k0, float* W, int ldw, float* d, float* e, float* tauq,
                float* taup) {
  const int C = tail_cluster_size(ctx);
  if (C == 0) return DDCSVD_ERR_UNSUPPORTED;
  TailParams p;
  p.mt = m - k0;
  p.nt = n - k0;
  p.ncb = ceil_div(p.nt, C);
  p.W = W + k0 + (size_t)k0 * ldw;
  p.ldw = ldw;
  p.d = d + k0;
  p.e = e + k0;
  p.tauq = tauq + k0;
  p.taup = taup + k0;
  const size_t smem = tail_smem_floats(p.mt, p.ncb) * sizeof(float);
  DDC_CUDA_TRY(cudaFuncSetAttribute((const void*)bidiag_tail_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(kTailThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  DDC_CUDA_TRY(cudaLaunchKernelEx(&cfg, bidiag_tail_kernel, p));
  count_launch();
  return DDCSVD_OK;
}

}  // namespace ddcsvd

#ifdef DDCSVD_PHASE_TRACE
extern "C" int ddcsvd_tail_trace_read(unsigned long long* out) {
  return (int)cudaMemcpyFromSymbol(out, ddcsvd::g_tail_trace, sizeof(ddcsvd::g_tail_trace));
}
#endif
