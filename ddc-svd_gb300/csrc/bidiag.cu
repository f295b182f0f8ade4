// bidiag.cu -- stage 1: Householder Golub-Kahan bidiagonalisation (FP32).
//
// Replaces bidiag_par (bidiag_par.c:34-450) and its ten OpenCL kernels
// (normsq_matcol/matrow, sum, update_scale_matcol/matrow, left/right_dotprods,
// left/right_update_mat, sanders).  Same reflector convention as the reference
// (bidiag.c:76-94): alpha_i = -sign(x_1) ||x||, sign(0) = +1, and a one-element
// reflector flips the sign (H = -1).  Reflectors are kept in LAPACK form in
// the working matrix (unit leading entry stored explicitly, scalar tau
// separate); export_reflectors() rewrites them in the reference's normalised
// form (H = I - 2 v v^T, ||v|| = 1).
//
// Two algorithms, both one persistent cooperative kernel per launch with a
// bounded grid barrier:
//
//  * bidiag_panel_kernel (BLOCKED modes): LAPACK-labrd-style panel of kPanel
//    columns.  Per column only the current column and row are updated; the
//    trailing block is read twice (y = A^T u, x = A v) and updated once per
//    panel by a rank-2*kPanel GEMM (tensor cores in the TF32X3/BF16X3 modes).
//    Work split: rows are owned by CTAs for column-shaped work (column update,
//    u scaling, x = A v, X), columns for row-shaped work (y = A^T u, Y, row
//    update, v scaling).  Because the GEMVs are fed with the *unscaled*
//    column/row (kept in xcol / xrow) and the reflector scale is applied
//    algebraically, each column costs exactly two grid barriers.  With up to
//    8192 rows the two GEMVs share one read of the trailing block: a CTA's
//    column dots are complete inside the CTA, so it knows the unscaled new
//    row values w of its columns within the pass and accumulates
//    sum_c A[r, c] w[c] for every row as it goes (one m-vector per CTA); the
//    row owners add the P vectors after the second barrier (the "fused"
//    pass -- the BLAS-2.5 idea of Howell et al., "Cache efficient
//    bidiagonalization using BLAS 2.5 operators", ACM TOMS 34(3), 2008).
//
//  * bidiag_plain_kernel (PLAIN_FP32): the reference's unblocked algorithm --
//    rank-1 update of the trailing block after every reflector
//    (left_update_mat.cl / right_update_mat.cl), fused with the dot products,
//    also two grid barriers per column.
//
// Loads of data that other CTAs write during the kernel go through L2 only
// (ld.global.cg) so that no SM reads a stale L1 line.
#include "internal.hpp"

namespace ddcsvd {

constexpr int kPS = 2 * kPanel + 4;  // floats per partial-sum record

#ifdef DDCSVD_PHASE_TRACE
__device__ unsigned long long g_phase_trace[128 * 16];
#endif
// phase marks of the panel kernel, CTA 7: column 5 of every panel (one row per
// panel), or with DDCSVD_TRACE_ALLCOLS every column of the panels at k0 = 0,
// 1024, 2048, 3072 (row = 32 * (k0 / 1024) + j)
// (slots 12 / 13: kernel entry / exit)
#ifdef DDCSVD_TRACE_ALLCOLS
#define PMARK(slot) DDC_MARK(blockIdx.x == 7 && (p.k0 & 1023) == 0, 32 * (p.k0 >> 10) + j, slot)
#define PMARK_K(slot) \
  DDC_MARK(blockIdx.x == 7 && (p.k0 & 1023) == 0, 32 * (p.k0 >> 10) + ((slot) == 12 ? 0 : 31), slot)
#else
#define PMARK(slot) DDC_MARK(blockIdx.x == 7 && j == 5, p.k0 / kPanel, slot)
#define PMARK_K(slot) DDC_MARK(blockIdx.x == 7, p.k0 / kPanel, slot)
#endif

struct PanelParams {
  int m, n, k0, nb, ldw, ldn, P;
  int rc, cc;  // rows / columns per CTA
  float* W;
  float *X, *Y, *VT;
  float *d, *e, *tauq, *taup;
  float *xcol, *xrow;
  float *colpart, *rowpart;  // [P][kPS]
  double *colnrm, *rownrm;   // [P]
  GridBarrier* bar;
  DevStatus* st;
  // tensor-core trailing update: the panel's [Up X] rows (>= k0 + nb) and
  // [Y VT] rows written K-major (2 * kPanel floats per row) at the end, or null
  float *Apk, *Bpk;
  // fused pass: float4 rows per thread (1, 2 or 4; 0 = two separate GEMVs)
  // and the per-CTA partial products x = A w ([P][ldxp], absolute row index)
  int rpt4;
  float* xpart;
  int ldxp;
  // two-GEMV form with more rows than shared memory holds next to the panel
  // blocks: y = A^T u reads the column from xcol (global, L2-resident)
  // instead of a staged copy, and the staging buffer holds only the row
  int ucol_global;
};

__device__ __forceinline__ float sgn_ref(float x) { return x < 0.f ? -1.f : 1.f; }

// Householder parameters for x = (x0, tail) with ||tail||^2 = t2 (FP64).
__device__ __forceinline__ void householder(float x0, double t2, float* alpha, float* tau,
                                            float* scale) {
  double nrm = sqrt((double)x0 * (double)x0 + t2);
  if (nrm == 0.0) {
    *alpha = 0.f;
    *tau = 0.f;
    *scale = 0.f;
    return;
  }
  double s = x0 < 0.f ? -1.0 : 1.0;
  double a = -s * nrm;
  *alpha = (float)a;
  *tau = (float)((nrm + fabs((double)x0)) / nrm);
  *scale = (float)(1.0 / ((double)x0 - a));
}

// sum_{r in [r0, r1)} col[r] * xs[r]; col in global (16B-aligned base), xs in
// shared memory indexed absolutely.  Warp-cooperative, result in all lanes.
// Eight 16-byte loads per lane are kept in flight.
// kGlobalX: xs is in global memory, written by other CTAs since this kernel
// started (read through L2, bypassing L1); otherwise shared memory.
template <bool kGlobalX = false>
__device__ __forceinline__ float warp_dot_col(const float* __restrict__ col, const float* xs, int r0,
                                              int r1, int lane) {
  float acc = 0.f;
  if (r1 <= r0) return 0.f;
  int a0 = min(r1, (r0 + 3) & ~3);
  int a1 = max(a0, r1 & ~3);
  auto xl = [&](int r) { return kGlobalX ? __ldcg(xs + r) : xs[r]; };
  auto xl4 = [&](const float4* v) { return kGlobalX ? __ldcg(v) : *v; };
  if (lane < a0 - r0) acc += __ldcg(col + r0 + lane) * xl(r0 + lane);
  if (lane < r1 - a1) acc += __ldcg(col + a1 + lane) * xl(a1 + lane);
  const float4* c4 = reinterpret_cast<const float4*>(col + a0);
  const float4* x4 = reinterpret_cast<const float4*>(xs + a0);
  const int nq = (a1 - a0) >> 2;
  int q = lane;
  for (; q + 224 < nq; q += 256) {
    float4 w[8];
#pragma unroll
    for (int u = 0; u < 8; u++) w[u] = __ldcg(c4 + q + 32 * u);
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const float4 v = xl4(x4 + q + 32 * u);
      acc += w[u].x * v.x + w[u].y * v.y + w[u].z * v.z + w[u].w * v.w;
    }
  }
  for (; q < nq; q += 32) {
    float4 w0 = __ldcg(c4 + q);
    float4 v0 = xl4(x4 + q);
    acc += w0.x * v0.x + w0.y * v0.y + w0.z * v0.z + w0.w * v0.w;
  }
  return warp_sum(acc);
}

// Row-block GEMV: out[r - ra] = sum_{c in [c0, n)} W[r, c] * xs[c] for the
// CTA's float4-aligned row block [ra, ra + 4*R4).  red: blockDim float4s.
// Each thread keeps eight 16-byte loads in flight.
__device__ __forceinline__ void block_rows_gemv(const float* __restrict__ W, int ldw, int ra,
                                                int R4, int c0, int n, const float* xs,
                                                float4* red, float* out) {
  const int t = threadIdx.x;
  const int G = blockDim.x / R4;
  const int q = t % R4, g = t / R4;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (g < G) {
    const float* base = W + ra + 4 * q;
    int c = c0 + g;
    for (; c + 7 * G < n; c += 8 * G) {
      float4 w[8];
#pragma unroll
      for (int u = 0; u < 8; u++)
        w[u] = __ldcg(reinterpret_cast<const float4*>(base + (size_t)(c + u * G) * ldw));
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const float x = xs[c + u * G];
        acc.x += w[u].x * x;
        acc.y += w[u].y * x;
        acc.z += w[u].z * x;
        acc.w += w[u].w * x;
      }
    }
    for (; c < n; c += G) {
      float4 w0 = __ldcg(reinterpret_cast<const float4*>(base + (size_t)c * ldw));
      float x0 = xs[c];
      acc.x += w0.x * x0;
      acc.y += w0.y * x0;
      acc.z += w0.z * x0;
      acc.w += w0.w * x0;
    }
  }
  red[t] = acc;
  __syncthreads();
  // pairwise tree over the G column groups (log2 G steps; a serial sum over
  // G = 512 groups of a 4-row block cost ~20 us per column)
  int half = 1;
  while (half < G) half <<= 1;
  for (half >>= 1; half > 0; half >>= 1) {
    if (g < half && g + half < G) {
      const float4 o = red[t + half * R4];
      float4 v = red[t];
      v.x += o.x;
      v.y += o.y;
      v.z += o.z;
      v.w += o.w;
      red[t] = v;
    }
    __syncthreads();
  }
  if (t < 4 * R4) {
    const float4 v = red[t >> 2];
    const int comp = t & 3;
    out[t] = comp == 0 ? v.x : comp == 1 ? v.y : comp == 2 ? v.z : v.w;
  }
  __syncthreads();
}

// Deterministic sum over the P per-CTA partial records of `cnt` floats plus
// the compensated norm pair at [kPS - 2], [kPS - 1].  Warp w takes records
// w, w + nw, ...; its lanes read each record along q (coalesced 128-byte
// lines: an earlier version read along b, one sector per lane, and its cost
// grew with cnt to ~9 us).  All loads of a warp are issued before the first
// add; the nw warp sums are then added in warp order, so the result does not
// depend on timing.  `red` holds nw * (kPS + 4) floats.
struct NoHook {
  __device__ void operator()() const {}
};

// `hook` runs in every thread after the thread's record loads have been
// consumed and before the first barrier: callers use it to store values they
// loaded into registers before the call, so that all loads of a phase share
// one round trip and the stores are visible after the reduction.
template <typename Hook = NoHook>
__device__ __forceinline__ void reduce_partials(const float* __restrict__ part, int P, int cnt, float* red,
                                                float* tot, FF* ntot, Hook hook = Hook()) {
  constexpr int kR = 12;  // records per warp held in one pass (P <= kR * nw in one pass)
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float a0 = 0.f, a1 = 0.f;
  FF nacc{0.f, 0.f};  // lane u < kR accumulates the norm pairs of the warp's u-th records
  for (int b0 = w; b0 < P; b0 += kR * nw) {
    float v0[kR], v1[kR];
#pragma unroll
    for (int u = 0; u < kR; u++) {
      const int b = b0 + u * nw;
      const float* rec = part + (size_t)b * kPS;
      const bool in = b < P;
      v0[u] = (in && lane < cnt) ? __ldcg(rec + lane) : 0.f;
      v1[u] = (in && lane + 32 < cnt) ? __ldcg(rec + 32 + lane) : 0.f;
    }
    const int bn = b0 + lane * nw;
    const float2 nv = (lane < kR && bn < P) ? __ldcg(reinterpret_cast<const float2*>(part + (size_t)bn * kPS + kPS - 2))
                                            : make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kR; u++) {
      a0 += v0[u];
      a1 += v1[u];
    }
    nacc = ff_add(nacc, FF{nv.x, nv.y});
  }
  nacc = warp_sum_ff(nacc);
  static_assert(2 * kPanel <= 64, "record entries beyond 64 are not reduced");
  float* rw = red + w * (kPS + 4);
  rw[lane] = a0;
  rw[32 + lane] = a1;
  if (lane == 0) {
    rw[kPS] = nacc.hi;
    rw[kPS + 1] = nacc.lo;
  }
  hook();
  __syncthreads();
  const int t = threadIdx.x;
  if (t < cnt && t < 64) {
    // four independent chains over the warps, added in a fixed order
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int k = 0;
    for (; k + 3 < nw; k += 4) {
      s0 += red[k * (kPS + 4) + t];
      s1 += red[(k + 1) * (kPS + 4) + t];
      s2 += red[(k + 2) * (kPS + 4) + t];
      s3 += red[(k + 3) * (kPS + 4) + t];
    }
    for (; k < nw; k++) s0 += red[k * (kPS + 4) + t];
    tot[t] = (s0 + s1) + (s2 + s3);
  } else if (t >= 64 && t < 96) {
    // the warp partials of the norm through one shuffle tree
    const int l = t - 64;
    FF v{0.f, 0.f};
    if (l < nw) v = FF{red[l * (kPS + 4) + kPS], red[l * (kPS + 4) + kPS + 1]};
    v = warp_sum_ff(v);
    if (l == 0) *ntot = v;
  }
  __syncthreads();
}

// Copies src[lo, hi) into the absolutely indexed shared buffer dst with
// 16-byte loads (dst and src share the same alignment; entries below lo in
// the first vector are copied too and never read).
__device__ __forceinline__ void stage_vec(float* dst, const float* __restrict__ src, int lo, int hi) {
  const int a = lo & ~3;
  const int nv = (hi - a + 3) >> 2;
  const float4* s4 = reinterpret_cast<const float4*>(src + a);
  float4* d4 = reinterpret_cast<float4*>(dst + a);
  for (int q = threadIdx.x; q < nv; q += blockDim.x) d4[q] = __ldcg(s4 + q);
}

constexpr int kLD = kPanel + 1;  // padded row length of the cached panel blocks

// Warp reduce-scatter of B per-lane values (B a power of two, at most 32):
// lane l returns the warp sum of v[l / (32 / B)].  Partners add in the order
// (own + received), which gives the same sum on both sides, so all 32 / B
// lanes of a group return the same value.  B - 1 + log2(32 / B) shuffles,
// against 5 B for B separate warp sums.
template <int B>
__device__ __forceinline__ float warp_reduce_scatter(float (&v)[B], int lane) {
#pragma unroll
  for (int nv = B, off = 16; nv > 1; nv >>= 1, off >>= 1) {
    const bool up = (lane & off) != 0;
#pragma unroll
    for (int h = 0; h < nv / 2; h++) {
      const float send = up ? v[h] : v[h + nv / 2];
      const float keep = up ? v[h + nv / 2] : v[h];
      v[h] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  float s = v[0];
#pragma unroll
  for (int off = 16 / B; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return s;
}

// Columns per batch of the fused pass for RPT4 float4 rows per thread (two
// batches of B * RPT4 float4s in registers).  Measured on the 4096^2 and
// 8192^2 factorisations: B * RPT4 = 4 at up to 4096 rows, B = 2 at up to 8192
// (the longer HBM latency of a matrix beyond L2 wants the deeper buffer).
__host__ __device__ constexpr int fused_cols(int rpt4) { return rpt4 <= 1 ? 4 : 2; }

// Fused column pass of S3.  Rows [sa, sa + 4 nq) are split over the threads
// in float4s (q = t + k * blockDim, k < RPT4: coalesced 512-byte lines per
// warp); the own columns [c_s, c_s + ncol) are taken B at a time, the next
// batch's loads issued into the second register buffer before the current
// batch is used.  Per batch: dots with the unscaled column xsb (zero outside
// rows [i+1, m)), a warp reduce-scatter and one block barrier, the new row
// value w of each column (Y column j, xrow, owncol as in the two-GEMV form),
// and acc[r] += W[r, c] w[c] for c >= i + 2 (column i + 1 enters x through
// its unit coefficient).  acc ends in xp (this CTA's record, absolute row
// index).  `prologue` runs after the first loads are issued, before a
// barrier.
template <int RPT4, int B, typename Prologue>
__device__ __forceinline__ void fused_col_pass(const float* __restrict__ W, int ldw, int m, int sa, int nq, int c_s,
                                               int ncol, int ca, int i, int j, const float* xsb, float* red,
                                               const float* c1s, const float* c2s, const float* pre, float tq,
                                               float sq, float* Y, int ldn, float* YS, float* owncol, float* xrow,
                                               float* xp, Prologue prologue) {
  constexpr int G = 32 / B;  // lanes per column after the reduce-scatter
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5, nt = blockDim.x;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  const int ns = (ncol + B - 1) / B;  // batches of this step
  // rows of the last float4 at or beyond m (padding of a caller's buffer may
  // hold anything) read as zero
  const int mt = m - sa - 4 * (nq - 1);  // valid rows of the last float4, 1..4
  auto msk = [&](float4 v, int k) {
    if (t + k * nt == nq - 1 && mt < 4) {
      if (mt < 2) v.y = 0.f;
      if (mt < 3) v.z = 0.f;
      v.w = 0.f;
    }
    return v;
  };
  float4 rA[B][RPT4], rB[B][RPT4];
  auto load = [&](float4(&dst)[B][RPT4], int s) {
#pragma unroll
    for (int u = 0; u < B; u++) {
      const bool cin = s * B + u < ncol;
      const float4* col = reinterpret_cast<const float4*>(W + (size_t)(cin ? c_s + s * B + u : c_s) * ldw + sa);
#pragma unroll
      for (int k = 0; k < RPT4; k++) {
        const int q = t + k * nt;
        dst[u][k] = (cin && q < nq) ? __ldcg(col + q) : z4;
      }
    }
  };
  if (ns > 0) load(rA, 0);
  float4 xs[RPT4], acc[RPT4];
#pragma unroll
  for (int k = 0; k < RPT4; k++) {
    const int q = t + k * nt;
    xs[k] = q < nq ? reinterpret_cast<const float4*>(xsb + sa)[q] : z4;
    acc[k] = z4;
  }
  prologue();
  __syncthreads();
  auto body = [&](float4(&cur)[B][RPT4], float4(&nxt)[B][RPT4], int s) {
    if (s + 1 < ns) load(nxt, s + 1);
    float pd[B];
#pragma unroll
    for (int u = 0; u < B; u++) {
      float a = 0.f;
#pragma unroll
      for (int k = 0; k < RPT4; k++) {
        const float4 v = msk(cur[u][k], k);
        a += v.x * xs[k].x + v.y * xs[k].y + v.z * xs[k].z + v.w * xs[k].w;
      }
      pd[u] = a;
    }
    const float ws = warp_reduce_scatter<B>(pd, lane);
    const int u = lane / G, sub = lane % G;
    float* rp = red + (s & 1) * (B * nw);  // [column][warp]
    if (sub == 0) rp[u * nw + wid] = ws;
    __syncthreads();
    float tot = 0.f;
    for (int w2 = sub; w2 < nw; w2 += G) tot += rp[u * nw + w2];
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, off);
    const int cl = s * B + u;
    float wv = 0.f;
    if (cl < ncol) {
      const float wic = pre[cl];
      const float ycj = tq * (wic + sq * tot - c1s[cl]);
      wv = wic - ycj - c2s[cl];
      if (wid == 0 && sub == 0) {
        const int c = c_s + cl;
        Y[c + (size_t)j * ldn] = ycj;
        YS[(c - ca) * kLD + j] = ycj;
        owncol[cl] = wv;
        xrow[c] = wv;
      }
      if (c_s + cl < i + 2) wv = 0.f;
    }
#pragma unroll
    for (int uu = 0; uu < B; uu++) {
      const float wb = __shfl_sync(0xffffffffu, wv, uu * G);
#pragma unroll
      for (int k = 0; k < RPT4; k++) {
        const float4 v = msk(cur[uu][k], k);
        acc[k].x += v.x * wb;
        acc[k].y += v.y * wb;
        acc[k].z += v.z * wb;
        acc[k].w += v.w * wb;
      }
    }
  };
  for (int s = 0; s < ns; s += 2) {
    body(rA, rB, s);
    if (s + 1 < ns) body(rB, rA, s + 1);
  }
  float4* xp4 = reinterpret_cast<float4*>(xp + sa);
#pragma unroll
  for (int k = 0; k < RPT4; k++) {
    const int q = t + k * nt;
    if (q < nq) xp4[q] = acc[k];
  }
}

// Shared-memory layout of the panel kernel (floats unless noted).
struct PanelSmem {
  float* big;     // max(m, n) + 4: xcol / xrow by absolute index
  float4* red;    // blockDim
  float* own;     // rc: own rows' x (S1) / GEMV output (S6)
  float* owncol;  // cc: own columns' updated row values
  float* ypart;   // cc * 8: column dot partials
  float* UpS;     // rc x kLD: own rows of the panel's left reflectors
  float* XS;      // rc x kLD: own rows of X
  float* YS;      // cc x kLD: own columns of Y
  float* VTS;     // cc x kLD: own columns of VT
  float* pre;     // max(rc, cc): prefetched original row/column entries
  float* misc;    // 8: prefetched scalars
  float *Yi, *VTi, *Wi, *Xi, *p1, *p2, *q1, *q2, *tot;
  FF* nrm;        // reduced compensated norm
  float* redp;    // (threads / 32) * (kPS + 4): per-warp partial sums
  float* scal;    // 8
  float* xr;      // fused pass: P * rc, the P partial products of the own rows
};

__device__ PanelSmem carve(float* smem, int bigsz, int rc, int cc, int P, bool fused) {
  PanelSmem s;
  float* p = smem;
  s.big = p;
  p += round_up(bigsz + 4, 4);
  s.red = reinterpret_cast<float4*>(p);
  p += 4 * blockDim.x;
  s.own = p;
  p += round_up(rc + 4, 4);
  s.owncol = p;
  p += round_up(cc + 4, 4);
  s.ypart = p;
  p += round_up(cc * 8 + 4, 4);
  s.UpS = p; p += rc * kLD;
  s.XS = p; p += rc * kLD;
  s.YS = p; p += cc * kLD;
  s.VTS = p; p += cc * kLD;
  s.pre = p; p += round_up(max(rc, cc) + 4, 4);
  s.misc = p; p += 8;
  s.Yi = p; p += kPanel + 4;
  s.VTi = p; p += kPanel + 4;
  s.Wi = p; p += kPanel + 4;
  s.Xi = p; p += kPanel + 4;
  s.p1 = p; p += kPanel + 4;
  s.p2 = p; p += kPanel + 4;
  s.q1 = p; p += kPanel + 4;
  s.q2 = p; p += kPanel + 4;
  s.tot = p; p += kPS + 4;
  p = reinterpret_cast<float*>(round_up(reinterpret_cast<uintptr_t>(p), 16));
  s.nrm = reinterpret_cast<FF*>(p);
  p += 64;
  s.scal = p;
  p += 8;
  s.redp = p;
  p += (blockDim.x / 32) * (kPS + 4);
  p = reinterpret_cast<float*>(round_up(reinterpret_cast<uintptr_t>(p), 16));
  s.xr = fused ? p : nullptr;
  return s;
}

size_t panel_smem_bytes(int bigsz, int rc, int cc, int threads, int P, bool fused) {
  size_t f = round_up(bigsz + 4, 4) + 4 * threads + round_up(rc + 4, 4) + round_up(cc + 4, 4) +
             round_up(cc * 8 + 4, 4) + 2 * (size_t)rc * kLD + 2 * (size_t)cc * kLD +
             round_up(std::max(rc, cc) + 4, 4) + 8 + 8 * (kPanel + 4) + kPS + 4 + 4 +
             64 + 8 + (size_t)(threads / 32) * (kPS + 4) + 4;
  if (fused) f += (size_t)P * rc;
  return f * sizeof(float) + 64;
}

// kRpt4 = p.rpt4: 0 the two-GEMV form, 1 / 2 / 4 the one-read form with that
// many float4 rows per thread.  One instantiation per form, each with its own
// register allocation.
template <int kRpt4>
__global__ void __launch_bounds__(kBidiagThreads, 1) bidiag_panel_kernel(PanelParams p) {
  extern __shared__ __align__(16) float smem[];
  const int m = p.m, n = p.n, k0 = p.k0, ldw = p.ldw, ldn = p.ldn;
  const int b = blockIdx.x, t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
  constexpr bool fx = kRpt4 > 0;
  PanelSmem S = carve(smem, p.ucol_global ? n : max(m, n), p.rc, p.cc, p.P, fx);
  float* W = p.W;
  float *X = p.X, *Y = p.Y, *VT = p.VT;
  // static partitions for this panel
  const int rbase = k0 & ~3;
  const int ra = rbase + b * p.rc, rb = min(m, ra + p.rc);
  const int ca = k0 + 1 + b * p.cc, cb = min(n, ca + p.cc);
  float prev_taup = 0.f;  // tau of the previous step's right reflector
  PMARK_K(12);

  for (int j = 0; j < p.nb; j++) {
    const int i = k0 + j;
    PMARK(0);
    // ---------------- S1: update column i on own rows, partial sums
    const int r_s = max(ra, i);
    const int nrow = max(0, rb - r_s);
    // Row i of Y (S.Yi), of VT (S.VTi) and the own rows of column i (S.pre,
    // indexed r - ra) were loaded by the previous step's S5; only the first
    // column of a panel loads here.  VT[i, j-1] is the previous right
    // reflector's unit leading element.
    if (j == 0) {
      for (int rr = t; rr < nrow; rr += blockDim.x) S.pre[r_s - ra + rr] = __ldcg(W + r_s + rr + (size_t)i * ldw);
    } else if (t == 0) {
      S.VTi[j - 1] = prev_taup != 0.f ? 1.f : 0.f;
    }
    __syncthreads();
    for (int rr = wid; rr < nrow; rr += nw) {  // warp per row, lanes over l
      const int r = r_s + rr, lr = r - ra;
      float part = 0.f;
      if (lane < j) part = S.UpS[lr * kLD + lane] * S.Yi[lane] + S.XS[lr * kLD + lane] * S.VTi[lane];
      part = warp_sum(part);
      if (lane == 0) {
        const float x = S.pre[lr] - part;
        S.own[rr] = x;
        p.xcol[r] = x;
      }
    }
    __syncthreads();
    {
      // partial sums over own rows r > i: [1..j] Up^T x, [1+j..2j] X^T x, and
      // ||x||^2 as a compensated pair at [kPS-2, kPS-1]
      const int r1 = max(r_s, i + 1);
      if (wid == 0) {
        FF acc{0.f, 0.f};
        for (int r = r1 + lane; r < rb; r += 32) acc = ff_add_sq(acc, S.own[r - r_s]);
        acc = warp_sum_ff(acc);
        if (lane == 0)
          *reinterpret_cast<float2*>(p.colpart + (size_t)b * kPS + kPS - 2) = make_float2(acc.hi, acc.lo);
      }
      if (t >= 32 && t < 32 + 2 * j) {
        const int q = t - 32;
        const float* src = (q < j) ? (S.UpS + q) : (S.XS + (q - j));
        float acc = 0.f;
        for (int r = r1; r < rb; r++) acc += src[(r - ra) * kLD] * S.own[r - r_s];
        p.colpart[(size_t)b * kPS + 1 + q] = acc;
      }
    }
    PMARK(1);
    if (!grid_sync(p.bar, p.P, p.st, 1)) return;
    PMARK(2);

    // ---------------- S2: column reflector
    // Every load of the phase (row i of the panel's W and X, x0, S3's inputs:
    // the unscaled column and row i of the own columns -- they do not depend
    // on the reflector -- and the partial records) is issued into registers
    // before any of them is used, so the phase costs one round trip; the
    // reduction's hook stores them to shared memory.
    const int c_s = max(ca, i + 1);
    const int ncol = max(0, cb - c_s);
    {
      float wi = 0.f, xi = 0.f, x0v = 0.f, pw = 0.f;
      if (t < j) {
        wi = __ldcg(W + i + (size_t)(k0 + t) * ldw);
        xi = __ldcg(X + i + (size_t)t * ldw);
      }
      if (t == 64) x0v = __ldcg(p.xcol + i);
      const bool stage = i < n - 1;
      const int sa = (i + 1) & ~3, snv = (stage && !p.ucol_global) ? (m - sa + 3) >> 2 : 0;
      const float4* src4 = reinterpret_cast<const float4*>(p.xcol + sa);
      float4* dst4 = reinterpret_cast<float4*>(S.big + sa);
      const int nt = blockDim.x;
      float4 sv0 = make_float4(0.f, 0.f, 0.f, 0.f), sv1 = sv0;
      if (t < snv) sv0 = __ldcg(src4 + t);
      if (t + nt < snv) sv1 = __ldcg(src4 + t + nt);
      if (stage && t < ncol) pw = __ldcg(W + i + (size_t)(c_s + t) * ldw);
      // entries outside rows [i+1, m) of the staged vectors are zeroed (the
      // fused pass multiplies whole float4s)
      auto msk = [&](int q, float4 v) {
        const int e = sa + 4 * q;
        if (e < i + 1 || e + 4 > m) {
          if (e < i + 1 || e >= m) v.x = 0.f;
          if (e + 1 < i + 1 || e + 1 >= m) v.y = 0.f;
          if (e + 2 < i + 1 || e + 2 >= m) v.z = 0.f;
          if (e + 3 < i + 1 || e + 3 >= m) v.w = 0.f;
        }
        return v;
      };
      reduce_partials(p.colpart, p.P, 2 * j + 1, S.redp, S.tot, S.nrm, [&]() {
        PMARK(14);
        if (t < j) {
          S.Wi[t] = wi;
          S.Xi[t] = xi;
        }
        if (t == 64) S.misc[0] = x0v;
        if (t < snv) dst4[t] = msk(t, sv0);
        if (t + nt < snv) dst4[t + nt] = msk(t + nt, sv1);
        if (stage && t < ncol) S.pre[t] = pw;
      });
      if (snv > 2 * nt || (stage && ncol > nt)) {  // very tall or wide panels: the rest in extra rounds
        for (int q = t + 2 * nt; q < snv; q += nt) dst4[q] = msk(q, __ldcg(src4 + q));
        if (stage)
          for (int cl = t + nt; cl < ncol; cl += nt) S.pre[cl] = __ldcg(W + i + (size_t)(c_s + cl) * ldw);
        __syncthreads();
      }
    }
    // every thread forms the reflector from the same shared inputs (no broadcast round)
    float tq, sq;
    {
      float alpha;
      householder_ff(S.misc[0], *S.nrm, &alpha, &tq, &sq);
      if (t == 0 && b == 0) {
        p.d[i] = alpha;
        p.tauq[i] = tq;
      }
    }
    if (t < j) {
      S.p1[t] = S.Wi[t] + sq * S.tot[1 + t];
      S.p2[t] = S.Xi[t] + sq * S.tot[1 + j + t];
    }
    for (int rr = t; rr < nrow; rr += blockDim.x) {
      const int r = r_s + rr;
      const float u = (r == i) ? 1.f : S.own[rr] * sq;
      W[r + (size_t)i * ldw] = u;
      S.UpS[(r - ra) * kLD + j] = u;
    }
    if (i == n - 1) break;  // last column: no right reflector
    PMARK(3);
    // ---------------- S3: y = A^T u on own columns, Y column j, row-i update
    if constexpr (fx) {
      // one pass over the own columns: y, w and the partial x = A w
      PMARK(4);
      float* c1s = S.ypart;
      float* c2s = S.ypart + p.cc;
      auto corr = [&]() {  // Y / VT corrections of y and of the row update, warp per column
        for (int cl = wid; cl < ncol; cl += nw) {
          const int lc = c_s + cl - ca;
          float a1 = 0.f, a2 = 0.f;
          if (lane < j) {
            const float yl = S.YS[lc * kLD + lane], vl = S.VTS[lc * kLD + lane];
            const float wl = S.Wi[lane], xl = S.Xi[lane];
            a1 = yl * (wl + sq * S.tot[1 + lane]) + vl * (xl + sq * S.tot[1 + j + lane]);
            a2 = yl * wl + vl * xl;
          }
          a1 = warp_sum(a1);
          a2 = warp_sum(a2);
          if (lane == 0) {
            c1s[cl] = a1;
            c2s[cl] = a2;
          }
        }
      };
      const int sa = (i + 1) & ~3, nq = (m - sa + 3) >> 2;
      float* xp = p.xpart + (size_t)b * p.ldxp;
      float* red = reinterpret_cast<float*>(S.red);
      constexpr int kR = fx ? kRpt4 : 1;
      fused_col_pass<kR, fused_cols(kR)>(W, ldw, m, sa, nq, c_s, ncol, ca, i, j, S.big, red, c1s, c2s, S.pre, tq, sq,
                                         Y, ldn, S.YS, S.owncol, p.xrow, xp, corr);
      PMARK(5);
    } else {
      PMARK(4);
      if (ncol > 0) {
        int segs = min(8, max(1, nw / ncol));
        const int len = m - (i + 1);
        const int seglen = (int)round_up(ceil_div(max(len, 1), segs), 4);
        for (int item = wid; item < ncol * segs; item += nw) {
          const int cl = item / segs, sg = item % segs;
          const int r0 = i + 1 + sg * seglen, r1 = min(m, r0 + seglen);
          float v = p.ucol_global ? warp_dot_col<true>(W + (size_t)(c_s + cl) * ldw, p.xcol, r0, r1, lane)
                                  : warp_dot_col(W + (size_t)(c_s + cl) * ldw, S.big, r0, r1, lane);
          if (lane == 0) S.ypart[cl * 8 + sg] = v;
        }
        __syncthreads();
        PMARK(5);
        for (int cl = wid; cl < ncol; cl += nw) {  // warp per column, lanes over l
          const int c = c_s + cl, lc = c - ca;
          float ydot = 0.f;
          for (int sg = 0; sg < segs; sg++) ydot += S.ypart[cl * 8 + sg];
          float c1 = 0.f, c2 = 0.f;
          if (lane < j) {
            const float yl = S.YS[lc * kLD + lane], vl = S.VTS[lc * kLD + lane];
            c1 = yl * S.p1[lane] + vl * S.p2[lane];
            c2 = yl * S.Wi[lane] + vl * S.Xi[lane];
          }
          c1 = warp_sum(c1);
          c2 = warp_sum(c2);
          if (lane == 0) {
            const float wic = S.pre[cl];
            const float ycj = tq * (wic + sq * ydot - c1);
            Y[c + (size_t)j * ldn] = ycj;
            S.YS[lc * kLD + j] = ycj;
            const float w = wic - ycj - c2;
            S.owncol[cl] = w;
            p.xrow[c] = w;
          }
        }
      }
    }
    {
      __syncthreads();
      // partials over own columns c > i+1: [1..j+1] Y^T w, [j+2..2j+1] VT^T w,
      // and ||w||^2 as a compensated pair at [kPS-2, kPS-1]
      const int c1 = max(c_s, i + 2);
      if (wid == 0) {
        FF acc{0.f, 0.f};
        for (int c = c1 + lane; c < cb; c += 32) acc = ff_add_sq(acc, S.owncol[c - c_s]);
        acc = warp_sum_ff(acc);
        if (lane == 0)
          *reinterpret_cast<float2*>(p.rowpart + (size_t)b * kPS + kPS - 2) = make_float2(acc.hi, acc.lo);
      }
      if (t >= 32 && t < 32 + 2 * j + 1) {
        const int q = t - 32;
        const float* src = (q <= j) ? (S.YS + q) : (S.VTS + (q - j - 1));
        float acc = 0.f;
        for (int c = c1; c < cb; c++) acc += src[(c - ca) * kLD] * S.owncol[c - c_s];
        p.rowpart[(size_t)b * kPS + 1 + q] = acc;
      }
    }
    PMARK(6);
    if (!grid_sync(p.bar, p.P, p.st, 2)) return;
    PMARK(7);

    // ---------------- S5: row reflector
    // One round trip, as in S2: x0 of the row, row i+1 of Y and VT (needed
    // below and, unscaled, by the next step's S1), S6's inputs (the unscaled
    // row and the original column i+1 of the own rows) and the records.
    {
      const int nt = blockDim.x;
      float x1v = 0.f, yiv = 0.f, vtv = 0.f, pc = 0.f;
      if (t == 64) x1v = __ldcg(p.xrow + i + 1);
      if (t >= 96 && t < 96 + j + 1) yiv = __ldcg(Y + i + 1 + (size_t)(t - 96) * ldn);
      if (t >= 160 && t < 160 + j) vtv = __ldcg(VT + i + 1 + (size_t)(t - 160) * ldn);
      const bool stage = !fx && i + 2 < n;  // the two-GEMV form stages the unscaled row for S6
      const int sa = (i + 2) & ~3, snv = stage ? (n - sa + 3) >> 2 : 0;
      const float4* src4 = reinterpret_cast<const float4*>(p.xrow + sa);
      float4* dst4 = reinterpret_cast<float4*>(S.big + sa);
      float4 sv0 = make_float4(0.f, 0.f, 0.f, 0.f), sv1 = sv0;
      if (t < snv) sv0 = __ldcg(src4 + t);
      if (t + nt < snv) sv1 = __ldcg(src4 + t + nt);
      const int r_lo = max(ra, i + 1);
      if (r_lo + t < rb) pc = __ldcg(W + r_lo + t + (size_t)(i + 1) * ldw);
      // fused pass: the P partial products of the own rows (float4 items
      // (record, q), rows below i + 1 skipped), into S.xr as [P][R4]
      constexpr int kXR = 5;
      const int R4 = fx ? max(0, (rb - ra + 3) >> 2) : 0;
      const int nxi = p.P * R4;
      float4* xr4 = reinterpret_cast<float4*>(S.xr);
      const int R4d = max(R4, 1);
      auto xload = [&](int it) {
        const int bq = it / R4d, q = it - bq * R4d;
        return (ra + 4 * q + 3 >= i + 1) ? __ldcg(reinterpret_cast<const float4*>(p.xpart + (size_t)bq * p.ldxp + ra) + q)
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
      };
      float4 xv[kXR];
#pragma unroll
      for (int u = 0; u < kXR; u++) xv[u] = (t + u * nt < nxi) ? xload(t + u * nt) : make_float4(0.f, 0.f, 0.f, 0.f);
      reduce_partials(p.rowpart, p.P, 2 * j + 2, S.redp, S.tot, S.nrm, [&]() {
        PMARK(15);
        if (t == 64) S.misc[1] = x1v;
        if (t >= 96 && t < 96 + j + 1) S.Yi[t - 96] = yiv;
        if (t >= 160 && t < 160 + j) S.VTi[t - 160] = vtv;
        if (t < snv) dst4[t] = sv0;
        if (t + nt < snv) dst4[t + nt] = sv1;
        if (r_lo + t < rb) S.pre[r_lo + t - ra] = pc;
#pragma unroll
        for (int u = 0; u < kXR; u++)
          if (t + u * nt < nxi) xr4[t + u * nt] = xv[u];
      });
      if (snv > 2 * nt || rb - r_lo > nt || nxi > kXR * nt) {  // very wide or tall panels: the rest in extra rounds
        for (int q = t + 2 * nt; q < snv; q += nt) dst4[q] = __ldcg(src4 + q);
        for (int r = r_lo + t + nt; r < rb; r += nt) S.pre[r - ra] = __ldcg(W + r + (size_t)(i + 1) * ldw);
        for (int it = t + kXR * nt; it < nxi; it += nt) xr4[it] = xload(it);
        __syncthreads();
      }
      if (fx) {
        // x of the own rows: the P records summed in record order, four
        // chains per row combined by a symmetric butterfly
        const int lr = t >> 2, h = t & 3;
        float sx = 0.f;
        if (lr < rb - ra)
          for (int bq = h; bq < p.P; bq += 4) sx += S.xr[bq * 4 * R4 + lr];
        sx += __shfl_xor_sync(0xffffffffu, sx, 1);
        sx += __shfl_xor_sync(0xffffffffu, sx, 2);
        if (lr < rb - ra && h == 0) S.own[lr] = sx;
      }
    }
    float tp, sp;
    {
      float beta;
      if (i < n - 2) {
        householder_ff(S.misc[1], *S.nrm, &beta, &tp, &sp);
      } else {  // one element left: no reflection (bidiag.c:125-129)
        beta = S.misc[1];
        tp = 0.f;
        sp = 0.f;
      }
      if (t == 0 && b == 0) {
        p.e[i] = beta;
        p.taup[i] = tp;
      }
    }
    prev_taup = tp;
    if (t <= j) S.q1[t] = S.Yi[t] + sp * S.tot[1 + t];
    if (t < j) S.q2[t] = S.VTi[t] + sp * S.tot[j + 2 + t];
    {
      const int c_s = max(ca, i + 1);
      for (int c = c_s + t; c < cb; c += blockDim.x) {
        float v;
        if (c == i + 1) v = (tp != 0.f) ? 1.f : 0.f;
        else v = S.owncol[c - c_s] * sp;
        W[i + (size_t)c * ldw] = v;
        VT[c + (size_t)j * ldn] = v;
        S.VTS[(c - ca) * kLD + j] = v;
      }
    }
    PMARK(8);
    __syncthreads();
    PMARK(9);
    // ---------------- S6: x = A v on own rows, X column j
    {
      const int r_lo = max(ra, i + 1);
      if (rb > r_lo) {
        const int R4 = (rb - ra + 3) >> 2;
        if (tp != 0.f && !fx) block_rows_gemv(W, ldw, ra, R4, i + 2, n, S.big, S.red, S.own);
        PMARK(10);
        for (int r = r_lo + wid; r < rb; r += nw) {  // warp per row, lanes over l
          const int lr = r - ra;
          float part = 0.f;
          if (lane <= j) part = S.UpS[lr * kLD + lane] * S.q1[lane];
          if (lane < j) part += S.XS[lr * kLD + lane] * S.q2[lane];
          part = warp_sum(part);
          if (lane == 0) {
            float xv = 0.f;
            if (tp != 0.f) xv = tp * (S.pre[lr] + sp * S.own[lr] - part);
            X[r + (size_t)j * ldw] = xv;
            S.XS[lr * kLD + j] = xv;
          }
        }
      }
    }
    __syncthreads();
    PMARK(11);
  }
  // K-major operands of the trailing update straight from the shared-memory
  // copies of the own rows / columns (replaces two pack kernels per panel)
  if (p.Apk) {
    const int kn = k0 + p.nb;
    constexpr int K2 = 2 * kPanel;
    const int r0 = max(ra, kn);
    for (int idx = t; idx < max(0, rb - r0) * K2; idx += blockDim.x) {
      const int r = r0 + idx / K2, jj = idx % K2, lr = r - ra;
      p.Apk[(size_t)(r - kn) * K2 + jj] = (jj < kPanel) ? S.UpS[lr * kLD + jj] : S.XS[lr * kLD + jj - kPanel];
    }
    const int c0 = max(ca, kn);
    for (int idx = t; idx < max(0, cb - c0) * K2; idx += blockDim.x) {
      const int c = c0 + idx / K2, jj = idx % K2, lc = c - ca;
      p.Bpk[(size_t)(c - kn) * K2 + jj] = (jj < kPanel) ? S.YS[lc * kLD + jj] : S.VTS[lc * kLD + jj - kPanel];
    }
  }
  PMARK_K(13);
}

// ------------------------------------------------------------------------
// Plain (unblocked) kernel: the whole bidiagonalisation in one launch.
// ------------------------------------------------------------------------
struct PlainParams {
  int m, n, ldw, P, rc, cc;
  float* W;
  float *d, *e, *tauq, *taup;
  float *xcol, *xrow;
  double *colnrm, *rownrm;
  GridBarrier* bar;
  DevStatus* st;
};

__global__ void __launch_bounds__(kBidiagThreads, 1) bidiag_plain_kernel(PlainParams p) {
  extern __shared__ __align__(16) float smem[];
  const int m = p.m, n = p.n, ldw = p.ldw;
  const int b = blockIdx.x, t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
  float* big = smem;
  float4* red = reinterpret_cast<float4*>(big + round_up(max(m, n) + 4, 4));
  float* own = reinterpret_cast<float*>(red + blockDim.x);
  float* owncol = own + round_up(p.rc + 4, 4);
  double* dred = reinterpret_cast<double*>(
      round_up(reinterpret_cast<uintptr_t>(owncol + round_up(p.cc + 4, 4)), 16));
  float* scal = reinterpret_cast<float*>(dred + 32);
  float* W = p.W;
  // fixed partitions for the whole factorisation
  const int ra = b * p.rc, rb = min(m, ra + p.rc);
  const int ca = 1 + b * p.cc, cb = min(n, ca + p.cc);
  // column 0 partials (the fused tail of S6 provides them for later columns)
  {
    const int r_s = max(ra, 0);
    double acc = 0.0;
    for (int r = r_s + t; r < rb; r += blockDim.x) {
      float x = __ldcg(W + r);
      p.xcol[r] = x;
      if (r > 0) acc += (double)x * x;
    }
    acc = block_sum(acc, dred);
    if (t == 0) p.colnrm[b] = acc;
  }
  if (!grid_sync(p.bar, p.P, p.st, 11)) return;
  for (int i = 0; i < n; i++) {
    // ---------------- column reflector
    if (t == 0) {
      double acc = 0.0;
      for (int bb = 0; bb < p.P; bb++) acc += __ldcg(p.colnrm + bb);
      float alpha, tau, scale;
      householder(__ldcg(p.xcol + i), acc, &alpha, &tau, &scale);
      scal[0] = alpha;
      scal[1] = tau;
      scal[2] = scale;
      if (b == 0) {
        p.d[i] = alpha;
        p.tauq[i] = tau;
      }
    }
    __syncthreads();
    const float tq = scal[1], sq = scal[2];
    for (int r = max(ra, i) + t; r < rb; r += blockDim.x)
      W[r + (size_t)i * ldw] = (r == i) ? 1.f : __ldcg(p.xcol + r) * sq;
    if (i == n - 1) break;
    // ---------------- left update of own columns (left_dotprods + left_update_mat)
    for (int r = i + 1 + t; r < m; r += blockDim.x) big[r] = __ldcg(p.xcol + r) * sq;
    if (t == 0) big[i] = 1.f;
    __syncthreads();
    {
      const int c_s = max(ca, i + 1);
      for (int c = c_s + wid; c < cb; c += nw) {
        float* col = W + (size_t)c * ldw;
        float wv = warp_dot_col(col, big, i, m, lane);
        const float f = tq * wv;
        for (int r = i + lane; r < m; r += 32) col[r] = __ldcg(col + r) - f * big[r];
        __syncwarp();
        if (lane == 0) {
          float v = __ldcg(col + i);
          owncol[c - c_s] = v;
          p.xrow[c] = v;
        }
      }
      __syncthreads();
      double acc = 0.0;
      for (int c = max(c_s, i + 2) + t; c < cb; c += blockDim.x) {
        double v = owncol[c - c_s];
        acc += v * v;
      }
      acc = block_sum(acc, dred);
      if (t == 0) p.rownrm[b] = acc;
    }
    if (!grid_sync(p.bar, p.P, p.st, 12)) return;
    // ---------------- row reflector
    if (t == 0) {
      double acc = 0.0;
      for (int bb = 0; bb < p.P; bb++) acc += __ldcg(p.rownrm + bb);
      float x0 = __ldcg(p.xrow + i + 1), beta, tau, scale;
      if (i < n - 2) householder(x0, acc, &beta, &tau, &scale);
      else { beta = x0; tau = 0.f; scale = 0.f; }
      scal[3] = beta;
      scal[4] = tau;
      scal[5] = scale;
      if (b == 0) {
        p.e[i] = beta;
        p.taup[i] = tau;
      }
    }
    __syncthreads();
    const float tp = scal[4], sp = scal[5];
    for (int c = max(ca, i + 1) + t; c < cb; c += blockDim.x)
      W[i + (size_t)c * ldw] = (c == i + 1) ? (tp != 0.f ? 1.f : 0.f) : __ldcg(p.xrow + c) * sp;
    for (int c = i + 2 + t; c < n; c += blockDim.x) big[c] = __ldcg(p.xrow + c) * sp;
    if (t == 0) big[i + 1] = 1.f;
    __syncthreads();
    // ---------------- right update of own rows (right_dotprods + right_update_mat)
    const int r_lo = max(ra, i + 1);
    double nacc = 0.0;
    if (rb > r_lo) {
      const int R4 = (rb - ra + 3) >> 2;
      if (tp != 0.f) {
        block_rows_gemv(W, ldw, ra, R4, i + 1, n, big, red, own);
        // own[r - ra] = sum_{c > i} W[r,c] v_c ; W[r, c] -= tp * own * v_c
        const int cols = n - (i + 1);
        for (int idx = t; idx < cols * (rb - r_lo); idx += blockDim.x) {
          const int cl = idx / (rb - r_lo), rr = idx % (rb - r_lo);
          const int r = r_lo + rr, c = i + 1 + cl;
          float* a = W + r + (size_t)c * ldw;
          *a = __ldcg(a) - tp * own[r - ra] * big[c];
        }
        __syncthreads();
      } else {
        __syncthreads();
        __syncthreads();
      }
      // fused: next column's partial norm on own rows
      for (int r = r_lo + t; r < rb; r += blockDim.x) {
        float x = __ldcg(W + r + (size_t)(i + 1) * ldw);
        p.xcol[r] = x;
        if (r > i + 1) nacc += (double)x * x;
      }
    }
    nacc = block_sum(nacc, dred);
    if (t == 0) p.colnrm[b] = nacc;
    if (!grid_sync(p.bar, p.P, p.st, 13)) return;
  }
}

// ------------------------------------------------------------------------
// Reflector export to the reference's storage (bidiag_par.c:63-68).
// ------------------------------------------------------------------------
__global__ void export_reflectors_kernel(int m, int n, const float* __restrict__ W, int ldw,
                                         const float* d, const float* e, const float* tauq,
                                         const float* taup, double* out) {
  const int c = blockIdx.x;
  for (int r = threadIdx.x; r < m; r += blockDim.x) {
    double v = 0.0;
    const float w = W[r + (size_t)c * ldw];
    if (r >= c) {  // left reflector c
      const float a = d[c], tq = tauq[c];
      double f = (a < 0.f ? 1.0 : -1.0) * sqrt(0.5 * (double)tq);
      v = f * (double)w;
      if (tq == 0.f) v = (r == c) ? 0.0 : 0.0;
    } else if (r == c - 1) {  // leading entry of right reflector r (or the no-reflect zero)
      const float tp = taup[r];
      v = (tp == 0.f) ? 0.0 : (e[r] < 0.f ? 1.0 : -1.0) * sqrt(0.5 * (double)tp) * (double)w;
    } else {  // r < c - 1: right reflector r
      const float tp = taup[r];
      v = (tp == 0.f) ? 0.0 : (e[r] < 0.f ? 1.0 : -1.0) * sqrt(0.5 * (double)tp) * (double)w;
    }
    out[r + (size_t)c * m] = v;
  }
}

// ------------------------------------------------------------------------
// Range scaling for the blocked path.  Its Householder norms are compensated
// FP32 sums, so the matrix is brought into [2^-40, 2^40] by an exact power of
// two when max|a| lies outside (LAPACK's xGESVD scales for the same reason);
// inputs already in range are not touched.  d and e are scaled back after the
// factorisation; the reflectors do not depend on the scale.
// ------------------------------------------------------------------------
__global__ void range_scan_kernel(int m, int n, const float* __restrict__ W, int ldw, unsigned* amax) {
  float mx = 0.f;
  const int m4 = m >> 2;
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const float4* col = reinterpret_cast<const float4*>(W + (size_t)c * ldw);
    for (int q = threadIdx.x; q < m4; q += blockDim.x) {
      const float4 v = col[q];
      mx = fmaxf(mx, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
    }
    for (int r = 4 * m4 + threadIdx.x; r < m; r += blockDim.x) mx = fmaxf(mx, fabsf(W[r + (size_t)c * ldw]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(amax, __float_as_uint(mx));
}

__global__ void range_apply_kernel(int m, int n, float* W, int ldw, const unsigned* amax) {
  const float s = range_scale(*amax);
  if (s == 1.f) return;
  for (int c = blockIdx.x; c < n; c += gridDim.x)
    for (int r = threadIdx.x; r < m; r += blockDim.x) W[r + (size_t)c * ldw] *= s;
}

__global__ void range_unscale_kernel(int n, float* d, float* e, const unsigned* amax) {
  const float s = range_scale(*amax);
  if (s == 1.f) return;
  const float inv = 1.f / s;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    d[i] *= inv;
    if (i < n - 1) e[i] *= inv;
  }
}

// ------------------------------------------------------------------------
// QR preprocessing of tall matrices (m >= 2n): Householder QR, panels of
// kPanel columns.  One persistent cooperative kernel per panel; CTAs own rows
// and keep their rows of the panel in shared memory for the whole panel.  Per
// column a single grid barrier: the reflector's dot products with the panel's
// remaining columns are formed from the unscaled column,
//   w_c = scale * sum_{r > i} x_r a_rc + a_ic,
// so the norm and the dots share one reduction; records and the published row
// i are double-buffered by column parity (a CTA can be at most one column
// ahead of any other).  Same reflector convention as the bidiagonalisation.
// ------------------------------------------------------------------------
struct QrParams {
  int m, k0, nb, ldw, P, rc;
  float* W;
  float* tau;
  float* Vp;  // masked unit-lower reflectors of the panel, rows k0.. (ld ldv)
  int ldv;
  float* part;  // [2][P][kPS]
  float* rowi;  // [2][kPanel + 4]: row i of the panel, published by its owner
  GridBarrier* bar;
  DevStatus* st;
};

size_t qr_smem_bytes(int rc, int threads) {
  return sizeof(float) * ((size_t)rc * kLD + (size_t)(threads / 32) * (kPS + 4) + kPS + 4 + kPanel + 4 + 16) + 64;
}

__global__ void __launch_bounds__(kBidiagThreads, 1) qr_panel_kernel(QrParams p) {
  extern __shared__ __align__(16) float smem[];
  const int t = threadIdx.x, wid = t >> 5, lane = t & 31, nw = blockDim.x >> 5, b = blockIdx.x;
  const int m = p.m, k0 = p.k0, nb = p.nb, ldw = p.ldw;
  const int ra = (k0 & ~3) + b * p.rc, rb = min(m, ra + p.rc);
  const int nrow = max(0, rb - ra);
  float* As = smem;  // own rows of the panel, [row][kLD]
  float* redp = As + (size_t)p.rc * kLD;
  float* tot = redp + nw * (kPS + 4);
  float* Ri = tot + kPS + 4;
  FF* nrm = reinterpret_cast<FF*>(reinterpret_cast<uintptr_t>(Ri + kPanel + 4 + 1) & ~(uintptr_t)7);
  float* W = p.W;
  for (int idx = t; idx < nrow * nb; idx += blockDim.x) {
    const int lr = idx % nrow, c = idx / nrow;
    As[lr * kLD + c] = W[ra + lr + (size_t)(k0 + c) * ldw];
  }
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    const int i = k0 + j;
    float* part = p.part + (size_t)(j & 1) * p.P * kPS;
    float* rowi = p.rowi + (j & 1) * (kPanel + 4);
    const int r1 = max(ra, i + 1);
    if (i >= ra && i < rb)  // the owner of row i publishes a_ic, c >= j
      for (int c = j + t; c < nb; c += blockDim.x) rowi[c] = As[(i - ra) * kLD + c];
    if (wid == 0) {
      FF acc{0.f, 0.f};
      for (int r = r1 + lane; r < rb; r += 32) acc = ff_add_sq(acc, As[(r - ra) * kLD + j]);
      acc = warp_sum_ff(acc);
      if (lane == 0) *reinterpret_cast<float2*>(part + (size_t)b * kPS + kPS - 2) = make_float2(acc.hi, acc.lo);
    } else if (t >= 32 && t < 32 + (nb - j - 1)) {
      const int c = j + 1 + (t - 32);
      float acc = 0.f;
      for (int r = r1; r < rb; r++) acc += As[(r - ra) * kLD + j] * As[(r - ra) * kLD + c];
      part[(size_t)b * kPS + (c - j - 1)] = acc;
    }
    if (!grid_sync(p.bar, p.P, p.st, 40)) return;
    if (t >= 64 && t < 64 + (nb - j)) Ri[t - 64] = __ldcg(rowi + j + (t - 64));  // Ri[0] = x0
    reduce_partials(part, p.P, nb - j - 1, redp, tot, nrm);
    float alpha, tq, sq;
    householder_ff(Ri[0], *nrm, &alpha, &tq, &sq);
    if (t == 0 && b == 0) p.tau[i] = tq;
    // columns c > j of the own rows r >= i (v_i = 1, v_r = scale x_r)
    for (int idx = t; idx < nrow * (nb - j - 1); idx += blockDim.x) {
      const int lr = idx % nrow, c = j + 1 + idx / nrow, r = ra + lr;
      if (r < i) continue;
      const float w = sq * tot[c - j - 1] + Ri[c - j];
      const float v = (r == i) ? 1.f : sq * As[lr * kLD + j];
      As[lr * kLD + c] -= tq * v * w;
    }
    __syncthreads();
    for (int lr = t; lr < nrow; lr += blockDim.x) {
      const int r = ra + lr;
      if (r == i) As[lr * kLD + j] = alpha;
      else if (r > i) As[lr * kLD + j] *= sq;
    }
    __syncthreads();
  }
  // write back; the masked reflectors go to Vp for the trailing update
  for (int idx = t; idx < nrow * nb; idx += blockDim.x) {
    const int lr = idx % nrow, c = idx / nrow, r = ra + lr;
    const float a = As[lr * kLD + c];
    W[r + (size_t)(k0 + c) * ldw] = a;
    if (r >= k0) p.Vp[(r - k0) + (size_t)c * p.ldv] = (r < k0 + c) ? 0.f : (r == k0 + c ? 1.f : a);
  }
}

__global__ void range_unscale_vec_kernel(int n, float* x, const unsigned* amax) {
  const float s = range_scale(*amax);
  if (s == 1.f) return;
  const float inv = 1.f / s;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] *= inv;
}

// ------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------
int bidiag_coop_ctas(ddcsvd_context* ctx, int m, int n) {
  (void)m;
  (void)n;
  return ctx->num_sms;
}

void plan_bidiag(Arena& a, int m, int n, int ldw, int P, GemmKind kind, BidiagWork* w) {
  w->ldn = (int)round_up(n, 32);
  w->P = P;
  w->X = a.take<float>((size_t)ldw * kPanel);
  w->Y = a.take<float>((size_t)w->ldn * kPanel);
  w->VT = a.take<float>((size_t)w->ldn * kPanel);
  w->xcol = a.take<float>(ldw + 4);
  w->xrow = a.take<float>(w->ldn + 4);
  w->colpart = a.take<float>((size_t)P * kPS + 2 * P);
  w->rowpart = a.take<float>((size_t)P * kPS + 2 * P);
  w->bar = a.take<GridBarrier>(4);
  w->amax = a.take<unsigned>(4);
  w->gemm_scratch = a.take<char>(gemm_scratch_bytes(kind, m, n, 2 * kPanel));
  const bool tc = (kind != GEMM_SIMT);
  w->Apk = a.take<float>(tc ? (size_t)m * 2 * kPanel + 64 : 16);
  w->Bpk = a.take<float>(tc ? (size_t)n * 2 * kPanel + 64 : 16);
  // partial products of the fused pass, when some panel has at most
  // kFusedRows rows from its first staged float4 down
  const int k0_last = ((n - 1) / kPanel) * kPanel;
  w->ldxp = ldw;
  w->xpart = (m - k0_last <= kFusedRows) ? a.take<float>((size_t)P * ldw + 4) : nullptr;
}

static int launch_coop(const void* fn, int P, int threads, size_t smem, void* args,
                       cudaStream_t s) {
  DDC_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  void* argv[] = {args};
  DDC_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(P), dim3(threads), argv, smem, s));
  count_launch();
  return DDCSVD_OK;
}

int bidiag_blocked(ddcsvd_context* ctx, int m, int n, float* W, int ldw, float* d, float* e,
                   float* tauq, float* taup, BidiagWork& w, GemmKind kind, Arena* scratch) {
  if (m < n || n <= 0) return DDCSVD_ERR_ARG;
  const int P = w.P;
  const int sg = std::min(n, 4 * ctx->num_sms);
  DDC_CUDA_TRY(cudaMemsetAsync(w.amax, 0, sizeof(unsigned), ctx->stream));
  range_scan_kernel<<<sg, 256, 0, ctx->stream>>>(m, n, W, ldw, w.amax);
  range_apply_kernel<<<sg, 256, 0, ctx->stream>>>(m, n, W, ldw, w.amax);
  count_launch(2);
  DDC_CUDA_TRY(cudaGetLastError());
  for (int k0 = 0; k0 < n; k0 += kPanel) {
    // the remaining columns on one thread-block cluster once they fit
    if (bidiag_tail_columns(ctx, m, n, k0) > 0) {
      ktimer_begin(ctx, KC_BIDIAG);
      DDC_TRY(bidiag_tail(ctx, m, n, k0, W, ldw, d, e, tauq, taup));
      ktimer_end(ctx);
      break;
    }
    const int nb = std::min(kPanel, n - k0);
    PanelParams pp;
    pp.m = m; pp.n = n; pp.k0 = k0; pp.nb = nb; pp.ldw = ldw; pp.ldn = w.ldn; pp.P = P;
    pp.rc = (int)round_up(ceil_div(m - (k0 & ~3), P), 4);
    pp.cc = std::max(1, ceil_div(n - k0 - 1, P));
    pp.W = W; pp.X = w.X; pp.Y = w.Y; pp.VT = w.VT;
    pp.d = d; pp.e = e; pp.tauq = tauq; pp.taup = taup;
    pp.xcol = w.xcol; pp.xrow = w.xrow;
    pp.colpart = w.colpart; pp.rowpart = w.rowpart;
    pp.colnrm = reinterpret_cast<double*>(w.colpart + (size_t)P * kPS);
    pp.rownrm = reinterpret_cast<double*>(w.rowpart + (size_t)P * kPS);
    // colnrm / rownrm live after the float records: make them 8-byte aligned
    pp.colnrm = reinterpret_cast<double*>(round_up(reinterpret_cast<uintptr_t>(pp.colnrm), 8));
    pp.rownrm = reinterpret_cast<double*>(round_up(reinterpret_cast<uintptr_t>(pp.rownrm), 8));
    pp.bar = w.bar;
    pp.st = ctx->d_status;
    const bool fused_pack = (kind != GEMM_SIMT) && nb == kPanel && k0 + nb < n;
    pp.Apk = fused_pack ? w.Apk : nullptr;
    pp.Bpk = fused_pack ? w.Bpk : nullptr;
    // one read of the trailing block per column when the rows fit 4 float4s
    // per thread (and a row owner's P records fit 4 lanes per row)
    {
      const int nq0 = (m - ((k0 + 1) & ~3) + 3) >> 2;
      int rpt4 = ceil_div(nq0, kBidiagThreads);
      if (rpt4 == 3) rpt4 = 4;
      const bool fuse = ctx->tune[TK_PANEL_FUSED] != 0 && w.xpart != nullptr && rpt4 <= 4 &&
                        4 * pp.rc <= kBidiagThreads;
      pp.rpt4 = fuse ? rpt4 : 0;
      pp.xpart = w.xpart;
      pp.ldxp = w.ldxp;
    }
    size_t smem = panel_smem_bytes(std::max(m, n), pp.rc, pp.cc, kBidiagThreads, P, pp.rpt4 > 0);
    pp.ucol_global = 0;
    if (smem > ctx->smem_optin && pp.rpt4 == 0) {
      pp.ucol_global = 1;
      smem = panel_smem_bytes(n, pp.rc, pp.cc, kBidiagThreads, P, false);
    }
    if (smem > ctx->smem_optin) {
      set_last_error("bidiagonalisation panel of %d x %d needs %zu bytes of shared memory per CTA (limit %zu): "
                     "too many rows for the direct path", m - k0, n - k0, smem, ctx->smem_optin);
      return DDCSVD_ERR_ARG;
    }
    DDC_CUDA_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBarrier), ctx->stream));
    ktimer_begin(ctx, KC_BIDIAG);
    const void* kfn = pp.rpt4 == 1   ? (const void*)bidiag_panel_kernel<1>
                      : pp.rpt4 == 2 ? (const void*)bidiag_panel_kernel<2>
                      : pp.rpt4 == 4 ? (const void*)bidiag_panel_kernel<4>
                                     : (const void*)bidiag_panel_kernel<0>;
    DDC_TRY(launch_coop(kfn, P, kBidiagThreads, smem, &pp, ctx->stream));
    ktimer_end(ctx);
    const int kn = k0 + nb;
    if (kn < n) {
      // W[kn:m, kn:n] -= U_p Y^T + X VT^T   (rank-2*nb update)
      const int M = m - kn, N = n - kn;
      Mat A1{W + kn + (size_t)k0 * ldw, 1, ldw};
      Mat B1{w.Y + kn, w.ldn, 1};  // B1(k, c) = Y[kn + c, k]
      Mat A2{w.X + kn, 1, ldw};
      Mat B2{w.VT + kn, w.ldn, 1};
      ktimer_begin(ctx, KC_TRAIL_GEMM);
      if (kind == GEMM_SIMT) {
        DDC_TRY(gemm(ctx, kind, M, N, nb, A1, B1, nb, A2, B2, -1.f, 1.f, W + kn + (size_t)kn * ldw,
                     ldw, scratch));
      } else {
        // tensor cores read K-major operands: [U_p X] and [Y VT] as rows of 2*nb
        // (written by the panel kernel itself for full panels)
        if (!fused_pack) {
          DDC_TRY(pack_kmajor(ctx, M, nb, W + kn + (size_t)k0 * ldw, ldw, nb, w.X + kn, ldw, w.Apk, 2 * kPanel));
          DDC_TRY(pack_kmajor(ctx, N, nb, w.Y + kn, w.ldn, nb, w.VT + kn, w.ldn, w.Bpk, 2 * kPanel));
        }
        DDC_TRY(gemm_tc_kmajor(ctx, kind, M, N, 2 * nb, w.Apk, 2 * kPanel, 0, w.Bpk, 2 * kPanel, 0,
                               W + kn + (size_t)kn * ldw, ldw, -1.f, 1.f, scratch));
      }
      ktimer_end(ctx);
    }
  }
  range_unscale_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(n, d, e, w.amax);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

int bidiag_plain(ddcsvd_context* ctx, int m, int n, float* W, int ldw, float* d, float* e,
                 float* tauq, float* taup, BidiagWork& w) {
  if (m < n || n <= 0) return DDCSVD_ERR_ARG;
  PlainParams pp;
  pp.m = m; pp.n = n; pp.ldw = ldw; pp.P = w.P;
  pp.rc = (int)round_up(ceil_div(m, w.P), 4);
  pp.cc = std::max(1, ceil_div(n - 1, w.P));
  pp.W = W; pp.d = d; pp.e = e; pp.tauq = tauq; pp.taup = taup;
  pp.xcol = w.xcol; pp.xrow = w.xrow;
  pp.colnrm = reinterpret_cast<double*>(round_up(reinterpret_cast<uintptr_t>(w.colpart), 8));
  pp.rownrm = reinterpret_cast<double*>(round_up(reinterpret_cast<uintptr_t>(w.rowpart), 8));
  pp.bar = w.bar;
  pp.st = ctx->d_status;
  DDC_CUDA_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBarrier), ctx->stream));
  size_t smem = (round_up(std::max(m, n) + 4, 4) + 4 * kBidiagThreads + round_up(pp.rc + 4, 4) +
                 round_up(pp.cc + 4, 4) + 4 + 64 + 16) * sizeof(float) + 64;
  if (smem > ctx->smem_optin) {
    set_last_error("the plain FP32 path stages a %d-entry column in shared memory (%zu bytes, limit %zu): "
                   "too many rows", std::max(m, n), smem, ctx->smem_optin);
    return DDCSVD_ERR_ARG;
  }
  ktimer_begin(ctx, KC_BIDIAG);
  int rc = launch_coop((const void*)bidiag_plain_kernel, w.P, kBidiagThreads, smem, &pp, ctx->stream);
  ktimer_end(ctx);
  return rc;
}

int range_scale_matrix(ddcsvd_context* ctx, int m, int n, float* W, int ldw, unsigned* amax) {
  const int sg = std::min(n, 4 * ctx->num_sms);
  DDC_CUDA_TRY(cudaMemsetAsync(amax, 0, sizeof(unsigned), ctx->stream));
  range_scan_kernel<<<sg, 256, 0, ctx->stream>>>(m, n, W, ldw, amax);
  range_apply_kernel<<<sg, 256, 0, ctx->stream>>>(m, n, W, ldw, amax);
  count_launch(2);
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

int range_unscale_vector(ddcsvd_context* ctx, int n, float* x, const unsigned* amax) {
  range_unscale_vec_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(n, x, amax);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

void plan_qr(Arena& a, int m, int n, int P, GemmKind kind, QrWork* w) {
  w->ldv = (int)round_up(m, 32);
  w->P = P;
  w->Vp = a.take<float>((size_t)w->ldv * kWideWY);  // the reflectors of one super-block
  w->UT = a.take<float>((size_t)m * kPanel + 64);
  w->W1s = a.take<float>((size_t)n * kPanel + 64);
  w->UTw = a.take<float>((size_t)m * kWideWY + 64);
  w->W1w = a.take<float>((size_t)n * kWideWY + 64);
  w->part = a.take<float>((size_t)2 * P * kPS + 64);
  w->rowi = a.take<float>(2 * (kPanel + 4));
  w->wys = a.take<float>(std::max(wy_block_scratch_floats(m), wy_wide_scratch_floats(m)));
  w->bar = a.take<GridBarrier>(4);
  w->gemm_scratch_bytes = gemm_scratch_bytes(kind, n, kWideWY, m);
  w->gemm_scratch = a.take<char>(w->gemm_scratch_bytes);
}

// Two-level blocking: super-blocks of kWideWY columns, each factored as
// kPanel-column panels (qr_panel_kernel) whose reflectors are applied at once
// only to the super-block's own remaining columns; the far trailing matrix is
// updated once per super-block with a kWideWY-reflector WY block (K = 128
// tensor-core products instead of four K = 32 passes over it).
int qr_blocked(ddcsvd_context* ctx, int m, int n, float* W, int ldw, float* tau, QrWork& w, GemmKind kind) {
  if (m < n || n <= 0) return DDCSVD_ERR_ARG;
  Arena sc;
  sc.base = w.gemm_scratch;
  sc.plan = false;
  sc.cap = w.gemm_scratch_bytes;
  for (int K0 = 0; K0 < n; K0 += kWideWY) {
    const int NB = std::min(kWideWY, n - K0);
    // reflector block of the super-block: column c = reflector K0 + c over
    // rows K0.. (zero above its unit entry)
    DDC_CUDA_TRY(cudaMemsetAsync(w.Vp, 0, sizeof(float) * (size_t)w.ldv * NB, ctx->stream));
    for (int k0 = K0; k0 < K0 + NB; k0 += kPanel) {
      const int nb = std::min(kPanel, K0 + NB - k0);
      const int off = k0 - K0;
      QrParams q;
      q.m = m; q.k0 = k0; q.nb = nb; q.ldw = ldw; q.P = w.P;
      q.rc = (int)round_up(ceil_div(m - (k0 & ~3), w.P), 4);
      q.W = W; q.tau = tau; q.Vp = w.Vp + off + (size_t)off * w.ldv; q.ldv = w.ldv;
      q.part = w.part; q.rowi = w.rowi; q.bar = w.bar; q.st = ctx->d_status;
      ktimer_begin(ctx, KC_QR);
      if (qr_smem_bytes(q.rc, kBidiagThreads) > ctx->smem_optin) {
        set_last_error("QR panel of %d rows needs %zu bytes of shared memory per CTA (limit %zu): too many rows",
                       m - k0, qr_smem_bytes(q.rc, kBidiagThreads), ctx->smem_optin);
        return DDCSVD_ERR_ARG;
      }
      DDC_CUDA_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBarrier), ctx->stream));
      DDC_TRY(launch_coop((const void*)qr_panel_kernel, w.P, kBidiagThreads, qr_smem_bytes(q.rc, kBidiagThreads), &q,
                          ctx->stream));
      ktimer_end(ctx);
      if (k0 + nb < K0 + NB) {
        // the super-block's remaining columns: W[k0:, k0+nb:K0+NB] := (I - V T^T V^T) W[...]
        const int rows = m - k0, ncols = K0 + NB - k0 - nb;
        const float* Vpan = w.Vp + (size_t)off * w.ldv;  // panel's reflectors, rows from K0
        ktimer_begin(ctx, KC_QR);
        DDC_TRY(wy_prepare_block(ctx, rows, nb, Vpan + off, w.ldv, tau + k0, w.UT, true, w.wys));
        DDC_TRY(gemm_tc_kmajor_t(ctx, kind, ncols, nb, rows, W + (size_t)(k0 + nb) * ldw, ldw, k0, Vpan, w.ldv, off,
                                 w.W1s, kPanel, 1.f, 0.f, &sc));
        DDC_TRY(gemm_tc_kmajor(ctx, kind, rows, ncols, nb, w.UT, kPanel, 0, w.W1s, kPanel, 0,
                               W + k0 + (size_t)(k0 + nb) * ldw, ldw, -1.f, 1.f, &sc));
        ktimer_end(ctx);
      }
    }
    if (K0 + NB < n) {
      // far trailing update: W[K0:, K0+NB:] := (I - V T^T V^T) W[K0:, K0+NB:]
      const int rows = m - K0, ncols = n - K0 - NB;
      ktimer_begin(ctx, KC_QR);
      DDC_TRY(wy_prepare_wide(ctx, rows, NB, w.Vp, w.ldv, tau + K0, w.UTw, true, w.wys));
      DDC_TRY(gemm_tc_kmajor_t(ctx, kind, ncols, NB, rows, W + (size_t)(K0 + NB) * ldw, ldw, K0, w.Vp, w.ldv, 0,
                               w.W1w, kWideWY, 1.f, 0.f, &sc));
      DDC_TRY(gemm_tc_kmajor(ctx, kind, rows, ncols, NB, w.UTw, kWideWY, 0, w.W1w, kWideWY, 0,
                             W + K0 + (size_t)(K0 + NB) * ldw, ldw, -1.f, 1.f, &sc));
      ktimer_end(ctx);
    }
  }
  return DDCSVD_OK;
}

int export_reflectors(ddcsvd_context* ctx, int m, int n, const float* W, int ldw, const float* d,
                      const float* e, const float* tauq, const float* taup, double* A_out) {
  export_reflectors_kernel<<<n, 256, 0, ctx->stream>>>(m, n, W, ldw, d, e, tauq, taup, A_out);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

}  // namespace ddcsvd

#ifdef DDCSVD_PHASE_TRACE
extern "C" int ddcsvd_trace_read(unsigned long long* out) {
  return (int)cudaMemcpyFromSymbol(out, ddcsvd::g_phase_trace, sizeof(ddcsvd::g_phase_trace));
}
#endif
