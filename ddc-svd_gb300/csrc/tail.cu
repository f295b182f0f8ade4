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
// one hardware cluster barrier per column: the right reflector's products
// x = A' v are gathered unscaled (v = e_1 + s * row, so x = A'(:, i+1) +
// s * A'(:, i+2:) row(i+2:)) right after the left update, every CTA adds the
// C partials for all rows itself, and since column i+1 after the right update
// is A'(:, i+1) - tau * x, every CTA also forms the next left reflector
// itself instead of waiting for the column's owner.  Reflector conventions, FP32 compensated
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
// (column-major, ld mt), u, x, xp[2], pc[2] [mt each; xp and pc, the ones
// other CTAs read, double-buffered by column parity], vrow [ncb], red [32 FF],
// scal [8], nrm [2 FF].
__host__ __device__ inline size_t tail_vec_floats(int mt) { return (size_t)((mt + 4 + 3) & ~3); }
__host__ __device__ inline size_t tail_smem_floats(int mt, int ncb) {
  return (((size_t)mt * ncb + 3) & ~(size_t)3) + 6 * tail_vec_floats(mt) + (((size_t)ncb + 3) & ~(size_t)3) +
         64 + 8 + 4;
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

// Right update of the own columns l >= lr with (tp, x, row i of A) and then
// their left update with (tq, u), rows > i, one warp per column: x and u for
// the lane's rows (i + 1 + lane + 32 j) in registers, each column read and
// written once.  Row i + 1 of the columns >= the local index lv is gathered
// into vrow for the next step.  Needs mt - i - 1 <= 32 KR.
template <int KR>
__device__ __forceinline__ void tail_fused_update(float* A, int mt, int i, int lr, int nown, float tp, float tq,
                                                  const float* x, const float* u, float* vrow, int lv) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int rb = i + 1 + lane;
  float uc[KR], xc[KR];
#pragma unroll
  for (int j = 0; j < KR; j++) {
    const int r = rb + 32 * j;
    uc[j] = r < mt ? u[r] : 0.f;
    xc[j] = (r < mt && tp != 0.f) ? x[r] : 0.f;  // x is not formed when tp = 0
  }
  for (int l = lr + wid; l < nown; l += nw) {
    float* col = A + (size_t)l * mt;
    const float f = tp * col[i];
    float c[KR];
    float y = 0.f;
#pragma unroll
    for (int j = 0; j < KR; j++) {
      const int r = rb + 32 * j;
      c[j] = r < mt ? col[r] - f * xc[j] : 0.f;
      y += uc[j] * c[j];
    }
    y = warp_sum(y) * tq;
#pragma unroll
    for (int j = 0; j < KR; j++) {
      const int r = rb + 32 * j;
      c[j] -= y * uc[j];
      if (r < mt) col[r] = c[j];
    }
    if (lane == 0 && l >= lv) vrow[l - lv] = c[0];
  }
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
  const size_t vec = tail_vec_floats(mt);
  float* A = sm;
  float* u = A + (((size_t)mt * ncb + 3) & ~(size_t)3);
  float* x = u + vec;
  float* xp = x + vec;      // [2][vec]
  float* pc = xp + 2 * vec;  // [2][vec]
  float* vrow = pc + 2 * vec;
  FF* red = reinterpret_cast<FF*>(vrow + ((ncb + 3) & ~3));
  float* scal = reinterpret_cast<float*>(red + 32);
  FF* nrm = reinterpret_cast<FF*>(scal + 8);  // [2]

  // Left reflector of column j from u[j..mt) (the column after every earlier
  // update).  Every CTA forms it from the same values in the same order, so
  // all hold the same u; the owner of column j also stores it there.
  auto form_left = [&](int j) {
    FF s2{0.f, 0.f};
    for (int r = j + 1 + t; r < mt; r += nt_) s2 = ff_add_sq(s2, u[r]);
    s2 = tail_sum_ff(s2, red);
    float alpha, tq, sq;
    householder_ff(u[j], s2, &alpha, &tq, &sq);
    __syncthreads();  // u[j] read by every thread before it is overwritten
    const bool own = j % C == rank;
    float* col = A + (size_t)(j / C) * mt;
    for (int r = j + t; r < mt; r += nt_) {
      const float v = (r == j) ? 1.f : u[r] * sq;
      u[r] = v;
      if (own) col[r] = v;
    }
    if (own && t == 0) {
      p.d[j] = alpha;
      p.tauq[j] = tq;
    }
    __syncthreads();
    return tq;
  };

  // Left update of the own columns > j with u (warp per column, in shared
  // memory); row j of the columns > j + 1 gathered into vrow.
  auto left_update = [&](int j, float tq) {
    const int l1 = lfirst(j + 1), l2 = lfirst(j + 2);
    for (int l = l1 + wid; l < nown; l += nw) {
      float* col = A + (size_t)l * mt;
      if (tq != 0.f) {
        float y = 0.f;
        for (int r = j + lane; r < mt; r += 32) y += u[r] * col[r];
        y = warp_sum(y) * tq;
        for (int r = j + lane; r < mt; r += 32) col[r] -= y * u[r];
      }
      if (lane == 0 && l >= l2) vrow[l - l2] = col[j];
    }
    __syncthreads();
  };

  // own columns into shared memory; column 0 to every CTA
  for (int l = 0; l < nown; l++)
    for (int r = t; r < mt; r += nt_) A[r + (size_t)l * mt] = p.W[r + (size_t)(rank + l * C) * p.ldw];
  for (int r = t; r < mt; r += nt_) u[r] = p.W[r];
  __syncthreads();
  left_update(0, form_left(0));
  cluster.sync();

  // step i: right reflector of row i, then the left reflector of column i + 1
  for (int i = 0; i + 1 < ncols; i++) {
    const int b = i & 1;
    float* xpb = xp + b * vec;
    float* pcb = pc + b * vec;
    const int l1 = lfirst(i + 1), l2 = lfirst(i + 2);
    const int own_next = (i + 1) % C;  // rank owning column i + 1
    TMARK(0);
    // ---- B: per row r > i the unscaled partial product of the right
    // reflector's x over the own columns >= i + 2, the partial squared norm of
    // row i over them, and column i + 1 copied (its owner replaces it in C
    // while the other CTAs still read it)
    {
      const int nz = nown - l2;
      const float* cnext = A + (size_t)((i + 1) / C) * mt;
      for (int r = i + 1 + t; r < mt; r += nt_) {
        const float* ar = A + r + (size_t)l2 * mt;
        float z = 0.f;
        for (int j = 0; j < nz; j++) z += ar[(size_t)j * mt] * vrow[j];
        xpb[r] = z;
      }
      if (rank == own_next)
        for (int r = i + t; r < mt; r += nt_) pcb[r] = cnext[r];
      if (wid == nw - 1) {
        FF s{0.f, 0.f};
        for (int j = lane; j < nz; j += 32) s = ff_add_sq(s, vrow[j]);
        s = warp_sum_ff(s);
        if (lane == 0) nrm[b] = s;
      }
    }
    TMARK(1);
    cluster.sync();  // partial norms, partial products and column i + 1 published
    TMARK(2);
    // ---- C: right reflector from row i (every CTA forms it; warp 0), and
    // x = a'(:, i+1) + sp * (sum of the C partial products) with the next
    // column a'(:, i+1) - tp * x, for all rows in every CTA: rows in aligned
    // groups of four (the vectors are padded past mt), four lanes per group
    // adding a quarter of the partials each
    const float* pn = cluster.map_shared_rank(pcb, own_next);
    const int r0 = (i + 1) & ~3;
    const int ngr = (mt - r0 + 3) >> 2;
    const int part = t & 3;
    auto right_reflector = [&](FF v, float x0) {  // warp 0; v: lane t < C holds CTA t's norm partial
      const FF tot = warp_sum_ff(v);
      float beta, tpv, spv;
      if (i < ncols - 2) {
        householder_ff(x0, tot, &beta, &tpv, &spv);
      } else {  // one element left: no reflection (bidiag.c:125-129)
        beta = x0;
        tpv = 0.f;
        spv = 0.f;
      }
      if (t == 0) {
        if (rank == 0) {
          p.e[i] = beta;
          p.taup[i] = tpv;
        }
        scal[1] = tpv;
        scal[2] = spv;
      }
    };
    auto zsum = [&](int r, bool load) {  // the group's rows summed over the C partials (all four lanes)
      float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      if (load) {
        for (int k = part; k < C; k += 4) {
          const float4 q = *reinterpret_cast<const float4*>(cluster.map_shared_rank(xpb, k) + r);
          z.x += q.x;
          z.y += q.y;
          z.z += q.z;
          z.w += q.w;
        }
      }
#pragma unroll
      for (int o = 1; o <= 2; o <<= 1) {  // sums commute: the four lanes agree bit for bit
        z.x += __shfl_xor_sync(0xffffffffu, z.x, o);
        z.y += __shfl_xor_sync(0xffffffffu, z.y, o);
        z.z += __shfl_xor_sync(0xffffffffu, z.z, o);
        z.w += __shfl_xor_sync(0xffffffffu, z.w, o);
      }
      return z;
    };
    auto finish = [&](int r, float4 a, float4 z, float tp, float sp) {  // x and the next column, rows r..r+3
      if (tp != 0.f) {
        const float4 xv = make_float4(a.x + sp * z.x, a.y + sp * z.y, a.z + sp * z.z, a.w + sp * z.w);
        *reinterpret_cast<float4*>(x + r) = xv;
        *reinterpret_cast<float4*>(u + r) =
            make_float4(a.x - tp * xv.x, a.y - tp * xv.y, a.z - tp * xv.z, a.w - tp * xv.w);
      } else {
        *reinterpret_cast<float4*>(u + r) = a;
      }
    };
    auto scale_row = [&](float tp, float sp) {  // row i of the own columns > i: the stored right reflector
      for (int l = l1 + t; l < nown; l += nt_) {
        float* a = A + i + (size_t)l * mt;
        *a = (rank + l * C == i + 1) ? (tp != 0.f ? 1.f : 0.f) : *a * sp;
      }
    };
    if (ngr <= (nt_ >> 2)) {
      // one group per four lanes covers every row: the partial sums are loaded
      // together with the reflector's inputs and wait in registers for tp and sp
      FF v{0.f, 0.f};
      float x0 = 0.f;
      if (t < 32) {
        if (t < C) v = cluster.map_shared_rank(nrm, t)[b];
        x0 = *cluster.map_shared_rank(pcb + i, own_next);
      }
      const int g = t >> 2;
      const bool act = g < ngr;
      const int r = r0 + 4 * g;
      const float4 z = zsum(r, act);
      const float4 a = (act && part == 0) ? *reinterpret_cast<const float4*>(pn + r) : make_float4(0.f, 0.f, 0.f, 0.f);
      if (t < 32) right_reflector(v, x0);
      __syncthreads();
      TMARK(3);
      const float tp = scal[1], sp = scal[2];
      scale_row(tp, sp);
      if (act && part == 0) finish(r, a, z, tp, sp);
    } else {
      if (t < 32) {
        const FF v = t < C ? cluster.map_shared_rank(nrm, t)[b] : FF{0.f, 0.f};
        right_reflector(v, *cluster.map_shared_rank(pcb + i, own_next));
      }
      __syncthreads();
      TMARK(3);
      const float tp = scal[1], sp = scal[2];
      scale_row(tp, sp);
      for (int g0 = 0; g0 < ngr; g0 += nt_ >> 2) {
        const int g = g0 + (t >> 2);
        const bool act = g < ngr;
        const int r = r0 + 4 * g;
        const float4 z = zsum(r, act && tp != 0.f);
        if (act && part == 0) finish(r, *reinterpret_cast<const float4*>(pn + r), z, tp, sp);
      }
    }
    __syncthreads();
    TMARK(4);
    const float tp = scal[1];
    const float tq = form_left(i + 1);
    TMARK(5);
    // ---- D: right update of the own columns > i + 1 (column i + 1 now holds
    // its left reflector), then their left update with it
    const int lr = lfirst(i + 2);
    const int rows = mt - i - 1;
    if (rows <= 32 * 16) {
      // one pass per column, x and u held in registers (the fewest per lane that hold the rows)
      const int lv = lfirst(i + 3);
      if (rows <= 32 * 4)
        tail_fused_update<4>(A, mt, i, lr, nown, tp, tq, x, u, vrow, lv);
      else if (rows <= 32 * 8)
        tail_fused_update<8>(A, mt, i, lr, nown, tp, tq, x, u, vrow, lv);
      else
        tail_fused_update<16>(A, mt, i, lr, nown, tp, tq, x, u, vrow, lv);
      __syncthreads();
    } else {
      if (tp != 0.f) {
        for (int r = i + 1 + t; r < mt; r += nt_) {
          const float f = tp * x[r];
          for (int l = lr; l < nown; l++) A[r + (size_t)l * mt] -= f * A[i + (size_t)l * mt];
        }
      }
      __syncthreads();
      left_update(i + 1, tq);
    }
    TMARK(6);
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
