// twisted.cu -- stages 3-4: singular vectors of the bidiagonal (FP64 core).
//
// Replaces CalcRightSingularVectors (parallel-twisted.c:554-637) and
// RighttoLeftSingularVectors (:530-551).  For each sigma_k the reference
// factors B^T B - sigma_k^2 I forward (P D1 P^T) and backward (Q D2 Q^T)
// (:320-362), picks the twist r = argmin |gamma| (:458-488), solves for the
// vector from x_r = 1 outwards (:494-521) and normalises it (:88-123).  It
// forms B^T B explicitly, which squares the condition number and fails on
// graded spectra.  Here the same two factorisations come from the
// differential stationary / progressive qd transforms of B^T B = L D L^T
// (d_i = a_i^2, l_i = b_i / a_i) taken from the bidiagonal itself, which keep
// relative accuracy for small sigma; twist, solve and normalisation follow
// the reference.  Left vectors: y = B x normalised (the reference divides by
// sigma, :548, which fails for sigma = 0).
//
// GB300 mapping: each lane owns one sigma_k; a CTA of four warps handles 32
// vectors: warp 0 runs the top-down (stationary) transform while warp 1 runs
// the bottom-up (progressive) transform of the same 32 shifts, then all four
// warps split the twist search and the norm passes by index segment and two
// of them solve the two halves of the twisted system concurrently.  Per-step arrays are stored
// interleaved by vector (element i of vector k at [i * N + k]) so every
// access of a warp is one contiguous 256-byte segment.
#include <vector>

#include "internal.hpp"
#include "prep.hpp"

namespace ddcsvd {

// max |a_i|, |b_i| as the bit pattern of a non-negative double (ordered like
// the value), for the floor below
__global__ void tw_absmax_kernel(int N, const double* __restrict__ a, const double* __restrict__ b,
                                 unsigned long long* amax) {
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    m = fmax(m, fabs(a[i]));
    if (i + 1 < N) m = fmax(m, fabs(b[i]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(amax, (unsigned long long)__double_as_longlong(m));
}

__global__ void tw_setup_kernel(int N, const double* __restrict__ a, const double* __restrict__ b,
                                const unsigned long long* amax, double* dd, double* ll, double* dl, double* dll) {
  // floor for zero diagonal entries (rank-deficient B): keeps l_i finite
  const double m = __longlong_as_double((long long)*amax);
  const double fl = (m > 0.0 ? m : 1.0) * DBL_EPSILON * DBL_EPSILON;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    double ai = a[i];
    if (fabs(ai) < fl) ai = (ai < 0.0) ? -fl : fl;
    const double di = ai * ai;
    const double li = (i + 1 < N) ? b[i] / ai : 0.0;
    dd[i] = di;
    ll[i] = li;
    dl[i] = di * li;
    dll[i] = di * li * li;
  }
}

struct TwParams {
  int N;
  const double *dd, *ll, *dl, *dll;
  const double* sigma;
  VecLayout L;
  double *Lp, *Um, *S, *Pp;  // compact block layout
  double* Z;
  double *xinv, *yinv;  // per vector
  int* rank;            // position of each vector within its group (ascending sigma)
  const double *a, *b;
};

constexpr int kTwWarps = 4;

// 32 vectors per CTA, one per lane; kTwWarps warps share the work of each
// vector: the stationary and progressive transforms run concurrently (warps
// 0 and 1), the twist search and ||B z|| are split over index segments
// (warp w takes segment w), and the two halves of the solve run concurrently
// (warp 0 below the twist, warp 1 above).
__global__ void __launch_bounds__(32 * kTwWarps) twisted_kernel(TwParams p) {
  __shared__ double s_val[kTwWarps][32];
  __shared__ int s_idx[kTwWarps][32];
  __shared__ double s_nrm[2][32];
  __shared__ int s_r[32];
  const int N = p.N;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  const bool act = k < N;
  const int lo = act ? p.L.blo[k] : 0, hi = act ? p.L.bhi[k] : 0;
  const int nb = hi - lo;
  const long long base = act ? p.L.base[k] + (k - lo) : 0;  // element i at base + (i - lo) * nb
  auto at = [&](int i) { return base + (long long)(i - lo) * nb; };
  const double lam = act ? p.sigma[k] * p.sigma[k] : 0.0;
  const double tiny = DBL_MIN / DBL_EPSILON;
  // The recurrences below are serial in their FP64 values but not in their
  // loads: every loop fetches its next kB inputs before the dependent chain
  // (one loop iteration per step waited a full memory round trip per step).
  constexpr int kB = 8;
  if (w == 0) {
    // stationary qd on the block: L D L^T - lam = L+ D+ L+^T, s_lo = -lam
    double s = -lam;
    for (int i0 = lo; i0 < hi - 1; i0 += kB) {
      double ddv[kB], dlv[kB], llv[kB];
#pragma unroll
      for (int u = 0; u < kB; u++) {
        const int i = min(i0 + u, hi - 2);
        ddv[u] = p.dd[i];
        dlv[u] = p.dl[i];
        llv[u] = p.ll[i];
      }
#pragma unroll
      for (int u = 0; u < kB; u++) {
        const int i = i0 + u;
        if (i < hi - 1) {
          double dp = ddv[u] + s;
          if (fabs(dp) < tiny) dp = -tiny;
          const double L = dlv[u] / dp;
          p.Lp[at(i)] = L;
          p.S[at(i)] = s;
          s = L * llv[u] * s - lam;
        }
      }
    }
    if (hi > lo) p.S[at(hi - 1)] = s;
  } else if (w == 1 && hi > lo) {
    // progressive qd on the block: L D L^T - lam = U- D- U-^T, p_{hi-1} = d_{hi-1} - lam
    double pv = p.dd[hi - 1] - lam;
    p.Pp[at(hi - 1)] = pv;
    for (int i0 = hi - 2; i0 >= lo; i0 -= kB) {
      double dllv[kB], ddv[kB], llv[kB];
#pragma unroll
      for (int u = 0; u < kB; u++) {
        const int i = max(i0 - u, lo);
        dllv[u] = p.dll[i];
        ddv[u] = p.dd[i];
        llv[u] = p.ll[i];
      }
#pragma unroll
      for (int u = 0; u < kB; u++) {
        const int i = i0 - u;
        if (i >= lo) {
          double dm = dllv[u] + pv;
          if (fabs(dm) < tiny) dm = -tiny;
          const double tt = ddv[u] / dm;
          p.Um[at(i)] = llv[u] * tt;
          pv = pv * tt - lam;
          p.Pp[at(i)] = pv;
        }
      }
    }
  }
  __syncthreads();
  // ---- twist index r = argmin |gamma_i|, gamma_i = s_i + p_i + lam; ties -> larger i
  {
    const int seg = (nb + kTwWarps - 1) / kTwWarps;
    const int a = lo + w * seg, b = min(hi, a + seg);
    double best = INFINITY;
    int bi = -1;
    for (int i0 = b - 1; i0 >= a; i0 -= kB) {  // downward scan, strict <: keeps the larger index on ties
      double sv[kB], pvv[kB];
#pragma unroll
      for (int u = 0; u < kB; u++) {
        const int i = max(i0 - u, a);
        sv[u] = p.S[at(i)];
        pvv[u] = p.Pp[at(i)];
      }
#pragma unroll
      for (int u = 0; u < kB; u++) {
        const int i = i0 - u;
        if (i >= a) {
          const double g = fabs(sv[u] + pvv[u] + lam);
          if (g < best) { best = g; bi = i; }
        }
      }
    }
    s_val[w][lane] = best;
    s_idx[w][lane] = bi;
  }
  __syncthreads();
  if (w == 0) {
    double best = INFINITY;
    int r = hi - 1;
    for (int q = kTwWarps - 1; q >= 0; q--) {  // segments from the top: the same order as one downward scan
      if (s_idx[q][lane] >= 0 && s_val[q][lane] < best) { best = s_val[q][lane]; r = s_idx[q][lane]; }
    }
    s_r[lane] = act ? r : 0;
  }
  __syncthreads();
  const int r = s_r[lane];
  // ---- solve N_r z = gamma_r e_r with z_r = 1, outwards from r (two directions in parallel)
  if (act && w == 0) {
    double z = 1.0, nrm = 1.0;
    p.Z[at(r)] = 1.0;
    for (int i0 = r - 1; i0 >= lo; i0 -= kB) {
      double lv[kB];
#pragma unroll
      for (int u = 0; u < kB; u++) lv[u] = p.Lp[at(max(i0 - u, lo))];
#pragma unroll
      for (int u = 0; u < kB; u++) {
        const int i = i0 - u;
        if (i >= lo) {
          z = -lv[u] * z;
          p.Z[at(i)] = z;
          nrm += z * z;
        }
      }
    }
    s_nrm[0][lane] = nrm;
  } else if (act && w == 1) {
    double z = 1.0, nrm = 0.0;
    for (int i0 = r + 1; i0 < hi; i0 += kB) {
      double uv[kB];
#pragma unroll
      for (int u = 0; u < kB; u++) uv[u] = p.Um[at(min(i0 + u, hi - 1) - 1)];
#pragma unroll
      for (int u = 0; u < kB; u++) {
        const int i = i0 + u;
        if (i < hi) {
          z = -uv[u] * z;
          p.Z[at(i)] = z;
          nrm += z * z;
        }
      }
    }
    s_nrm[1][lane] = nrm;
  }
  __syncthreads();
  // ---- ||B z||^2 for the left vector, split by segment (b is zero at the block end)
  {
    double by = 0.0;
    if (act) {
      const int seg = (nb + kTwWarps - 1) / kTwWarps;
      const int a = lo + w * seg, b = min(hi, a + seg);
#pragma unroll 8
      for (int i = a; i < b; i++) {
        const double zi = p.Z[at(i)];
        const double zn = (i + 1 < hi) ? p.Z[at(i + 1)] : 0.0;
        const double y = p.a[i] * zi + ((i + 1 < hi) ? p.b[i] * zn : 0.0);
        by += y * y;
      }
    }
    s_val[w][lane] = by;
  }
  __syncthreads();
  if (w == 0 && act) {
    double by = 0.0;
    for (int q = 0; q < kTwWarps; q++) by += s_val[q][lane];
    p.xinv[k] = 1.0 / sqrt(s_nrm[0][lane] + s_nrm[1][lane]);
    p.yinv[k] = (by > 0.0) ? 1.0 / sqrt(by) : 0.0;
  }
}

// ---- clusters of (numerically) equal singular values inside one block
// The twisted solve of sigma_k is accurate to about eps * sigma_max / gap, so
// values that coincide to working precision inside one unreduced block get
// the same vector from it (the reference assumes distinct values,
// Calculations-Parallel.c:43).  Runs of sigmas closer than kClusterRel *
// sigma_max get their vectors from a shared subspace instead: distinct
// starts (the twisted vector plus a fixed pseudo-random vector), three steps
// of inverse iteration with the run's mid shift, and modified Gram-Schmidt
// (against the singleton neighbours, then the earlier members) after each
// step, as LAPACK's xSTEIN does for close eigenvalues.  Any orthonormal basis
// of the cluster's right singular subspace is a valid set of vectors when the
// values coincide; when they differ by less than the threshold the mixing
// adds at most that difference to the residual.  Singletons are untouched.
constexpr double kClusterRel = 1e-10;
constexpr int kClThreads = 256;

// deterministic value in [-1, 1) from (i, j): integer mixing (xorshift-multiply)
__device__ __forceinline__ double cl_start(int i, int j) {
  unsigned h = (unsigned)i * 0x9E3779B1u ^ ((unsigned)j * 0x85EBCA77u + 0x165667B1u);
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return (double)(h >> 8) * (2.0 / 16777216.0) - 1.0;
}

__device__ __forceinline__ double cl_block_max(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double r = 0.0;
  for (int q = 0; q < nw; q++) r = fmax(r, red[q]);
  return r;
}

// slot k starts a run of at least two close values
__device__ __forceinline__ bool cl_leader(const TwParams& p, int k) {
  const int lo = p.L.blo[k], hi = p.L.bhi[k];
  if (hi - lo < 2 || k + 1 >= hi) return false;
  const double* sg = p.sigma;  // ascending within the block
  const double smax = fabs(sg[hi - 1]);
  const double tol = kClusterRel * smax;
  return smax > 0.0 && (k == lo || sg[k] - sg[k - 1] > tol) && sg[k + 1] - sg[k] <= tol;
}

__device__ void cl_refine(const TwParams& p, int k0, double* red);

// each thread tests one slot; the CTA then refines the runs that start in
// its chunk (runs are independent, so their order does not matter)
__global__ void __launch_bounds__(kClThreads) tw_cluster_kernel(TwParams p) {
  __shared__ double red[kClThreads / 32];
  __shared__ int s_list[kClThreads];
  __shared__ int s_cnt;
  const int N = p.N, t = threadIdx.x, nt = blockDim.x;
  for (int c0 = blockIdx.x * nt; c0 < N; c0 += gridDim.x * nt) {
    if (t == 0) s_cnt = 0;
    __syncthreads();
    if (c0 + t < N && cl_leader(p, c0 + t)) s_list[atomicAdd(&s_cnt, 1)] = c0 + t;
    __syncthreads();
    const int cnt = s_cnt;
    for (int q = 0; q < cnt; q++) cl_refine(p, s_list[q], red);
    __syncthreads();
  }
}

__device__ void cl_refine(const TwParams& p, int k0, double* red) {
  const int t = threadIdx.x, nt = blockDim.x;
  {
    const int lo = p.L.blo[k0], hi = p.L.bhi[k0], nb = hi - lo;
    const double* sg = p.sigma;
    const double smax = fabs(sg[hi - 1]);
    const double tol = kClusterRel * smax;
    int c = 2;
    while (k0 + c < hi && sg[k0 + c] - sg[k0 + c - 1] <= tol) c++;
    const long long base = p.L.base[lo];
    const long long zc = base + (k0 - lo);  // Z column of member 0, element i at zc + j + (i - lo) * nb
    // contiguous work rows (free after the twisted solve; clusters own disjoint rows)
    double* W = p.Um + base + (long long)(k0 - lo) * nb;  // member j, element i at W[j * nb + i - lo]
    double* Lf = p.Pp + base + (long long)(k0 - lo) * nb;
    double* Df = Lf + nb;
    // neighbours that are singletons (their vectors are accurate and final)
    const int kl = (k0 > lo && (k0 - 1 == lo || sg[k0 - 1] - sg[k0 - 2] > tol)) ? k0 - 1 : -1;
    const int kr = (k0 + c < hi && (k0 + c + 1 == hi || sg[k0 + c + 1] - sg[k0 + c] > tol)) ? k0 + c : -1;
    // L+ D+ L+^T = (B^T B - lam I) / smax^2 by the stationary qd transform,
    // pivots kept at least 4 eps away from zero
    if (t == 0) {
      const double is = 1.0 / smax;
      const double sm = 0.5 * (sg[k0] + sg[k0 + c - 1]) * is;
      const double lam = sm * sm, fl = 4.0 * DBL_EPSILON;
      double s = -lam;
      for (int i = lo; i < hi; i++) {
        double dp = p.dd[i] * is * is + s;
        if (fabs(dp) < fl) dp = (dp < 0.0) ? -fl : fl;
        Df[i - lo] = dp;
        if (i + 1 < hi) {
          const double L = p.dl[i] * is * is / dp;
          Lf[i - lo] = L;
          s = L * p.ll[i] * s - lam;
        }
      }
    }
    const double rs = rsqrt((double)nb);
    for (long long q = t; q < (long long)c * nb; q += nt) {  // c * nb may pass 2^31 on huge blocks
      const int j = (int)(q / nb), i = lo + (int)(q % nb);
      W[q] = p.Z[zc + j + (long long)(i - lo) * nb] * p.xinv[k0 + j] + cl_start(i, j) * rs;
    }
    __syncthreads();
    for (int it = 0; it < 3; it++) {
      // inverse iteration: W_j <- (L+ D+ L+^T)^{-1} W_j, one thread per member
      for (int j = t; j < c; j += nt) {
        double* w = W + (long long)j * nb;
        double u = 0.0;
        for (int i = 0; i < nb; i++) {
          u = w[i] - (i > 0 ? Lf[i - 1] * u : 0.0);
          w[i] = u;
        }
        double z = 0.0;
        for (int i = nb - 1; i >= 0; i--) {
          z = w[i] / Df[i] - (i + 1 < nb ? Lf[i] * z : 0.0);
          w[i] = z;
        }
      }
      __syncthreads();
      // modified Gram-Schmidt, members in order; every thread keeps the same
      // elements i throughout, so the updates need no barrier of their own
      for (int j = 0; j < c; j++) {
        double* w = W + (long long)j * nb;
        double mx = 0.0;
        for (int i = t; i < nb; i += nt) mx = fmax(mx, fabs(w[i]));
        mx = cl_block_max(mx, red);
        if (mx > 0.0 && mx < INFINITY) {
          const double sc = 1.0 / mx;
          for (int i = t; i < nb; i += nt) w[i] *= sc;
        }
        for (int side = 0; side < 2; side++) {
          const int kn = side ? kr : kl;
          if (kn < 0) continue;
          const long long zn = base + (kn - lo);
          const double xn = p.xinv[kn];
          double d = 0.0;
          for (int i = t; i < nb; i += nt) d += w[i] * p.Z[zn + (long long)i * nb] * xn;
          d = block_sum(d, red);
          for (int i = t; i < nb; i += nt) w[i] -= d * p.Z[zn + (long long)i * nb] * xn;
        }
        for (int l = 0; l < j; l++) {
          const double* v = W + (long long)l * nb;
          double d = 0.0;
          for (int i = t; i < nb; i += nt) d += w[i] * v[i];
          d = block_sum(d, red);
          for (int i = t; i < nb; i += nt) w[i] -= d * v[i];
        }
        double n2 = 0.0;
        for (int i = t; i < nb; i += nt) n2 += w[i] * w[i];
        n2 = block_sum(n2, red);
        const double inv = (n2 > 0.0) ? 1.0 / sqrt(n2) : 0.0;
        for (int i = t; i < nb; i += nt) w[i] *= inv;
      }
      __syncthreads();
    }
    // back into the compact layout; unit norm, and 1 / ||B x|| for the left vector
    for (int j = 0; j < c; j++) {
      const double* w = W + (long long)j * nb;
      double by = 0.0;
      for (int i = t; i < nb; i += nt) {
        const double y = p.a[lo + i] * w[i] + (i + 1 < nb ? p.b[lo + i] * w[i + 1] : 0.0);
        by += y * y;
        p.Z[zc + j + (long long)i * nb] = w[i];
      }
      by = block_sum(by, red);
      if (t == 0) {
        p.xinv[k0 + j] = 1.0;
        p.yinv[k0 + j] = (by > 0.0) ? 1.0 / sqrt(by) : 0.0;
      }
    }
    __syncthreads();
  }
}

// rank of sigma_k among the sigmas of its group (ascending, stable):
// rank_k = #{j in group : s_j < s_k or (s_j == s_k and j < k)}.  The count
// is split over slot segments (grid y) so that a single large group (one SVD:
// N^2 comparisons) spreads over the whole GPU; each CTA stages the part of
// its segment that its threads' groups touch in shared memory, and adds its
// partial counts with integer atomics (rank zeroed beforehand), so the
// result is exact and independent of the order.
constexpr int kRankThreads = 256;
constexpr int kRankTile = 1024;

__global__ void __launch_bounds__(kRankThreads) tw_rank_count_kernel(int N, const double* __restrict__ sigma,
                                                                   VecLayout L, int* rank, int seg) {
  __shared__ double tile[kRankTile];
  __shared__ int s_lo, s_hi;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  int glo = N, ghi = 0;
  double v = 0.0;
  if (k < N) {
    const int g = L.grp[k];
    glo = L.g_lo[g];
    ghi = glo + L.g_n[g];
    v = sigma[k];
  }
  if (threadIdx.x == 0) {
    s_lo = N;
    s_hi = 0;
  }
  __syncthreads();
  if (k < N) {
    atomicMin(&s_lo, glo);
    atomicMax(&s_hi, ghi);
  }
  __syncthreads();
  const int j0 = max(blockIdx.y * seg, s_lo), j1 = min(min(N, (blockIdx.y + 1) * seg), s_hi);
  int cnt = 0;
  for (int t0 = j0; t0 < j1; t0 += kRankTile) {
    const int t1 = min(j1, t0 + kRankTile);
    for (int j = t0 + threadIdx.x; j < t1; j += blockDim.x) tile[j - t0] = sigma[j];
    __syncthreads();
    const int a = max(t0, glo), b = min(t1, ghi);
    for (int j = a; j < b; j++) {
      const double u = tile[j - t0];
      cnt += (u < v) || (u == v && j < k);
    }
    __syncthreads();
  }
  if (k < N && cnt) atomicAdd(&rank[k], cnt);
}

__global__ void tw_rank_place_kernel(int N, const double* __restrict__ sigma, VecLayout L, const int* rank,
                                     double* sorted) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x)
    sorted[L.g_lo[L.grp[k]] + rank[k]] = sigma[k];
}

static int rank_values(ddcsvd_context* ctx, int N, const double* sigma, const VecLayout& L, int* rank,
                       double* sorted) {
  DDC_CUDA_TRY(cudaMemsetAsync(rank, 0, sizeof(int) * (size_t)N, ctx->stream));
  const int nseg = std::max(1, std::min(16, ceil_div(N, 512)));
  const int seg = ceil_div(N, nseg);
  tw_rank_count_kernel<<<dim3(ceil_div(N, kRankThreads), nseg), kRankThreads, 0, ctx->stream>>>(N, sigma, L, rank,
                                                                                                  seg);
  count_launch();
  if (sorted) {
    tw_rank_place_kernel<<<std::min(ceil_div(N, 256), 8 * ctx->num_sms), 256, 0, ctx->stream>>>(N, sigma, L, rank,
                                                                                                sorted);
    count_launch();
  }
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

// One 32 x 32 tile (vectors k0.., rows i0.. of a block) per CTA:
// X[i - g0 + rank_k * ldx] = z_k[i] / ||z_k||, Y[...] = (B z_k)[i] / ||B z_k||
// (rows are local to the group; rows outside the block are zero).
__global__ void tw_finalize_kernel(TwParams p) {
  __shared__ double tile[33][33];
  const int4 T = p.L.tiles[blockIdx.x];
  const int lo = T.x, nb = T.y, k0 = lo + T.z, i0 = lo + T.w, hi = lo + nb;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  const long long base = p.L.base[lo];
  for (int rr = ty; rr < 33; rr += 8) {
    const int i = i0 + rr, k = k0 + tx;
    tile[rr][tx] = (i < hi && k < hi) ? p.Z[base + (long long)(i - lo) * nb + (k - lo)] : 0.0;
  }
  __syncthreads();
  for (int kk = ty; kk < 32; kk += 8) {
    const int k = k0 + kk, i = i0 + tx;
    if (k >= hi || i >= hi) continue;
    const int g = p.L.grp[k];
    const int g0 = p.L.g_lo[g];
    const int col = p.rank[k];
    const double xi = tile[tx][kk], xn = tile[tx + 1][kk];
    p.L.g_X[g][(i - g0) + (size_t)col * p.L.g_ldx[g]] = (float)(xi * p.xinv[k]);
    const double y = p.a[i] * xi + ((i + 1 < hi) ? p.b[i] * xn : 0.0);
    p.L.g_Y[g][(i - g0) + (size_t)col * p.L.g_ldy[g]] = (float)(y * p.yinv[k]);
  }
}

// zero the rows of each output column that lie outside the vector's block
__global__ void tw_zero_outside_kernel(int N, TwParams p) {
  for (int k = blockIdx.x; k < N; k += gridDim.x) {
    const int g = p.L.grp[k], g0 = p.L.g_lo[g], gn = p.L.g_n[g];
    const int lo = p.L.blo[k], hi = p.L.bhi[k];
    if (hi - lo == gn) continue;
    const int col = p.rank[k];
    float* X = p.L.g_X[g] + (size_t)col * p.L.g_ldx[g];
    float* Y = p.L.g_Y[g] + (size_t)col * p.L.g_ldy[g];
    for (int i = threadIdx.x; i < gn; i += blockDim.x) {
      const int gi = g0 + i;
      if (gi < lo || gi >= hi) {
        X[i] = 0.f;
        Y[i] = 0.f;
      }
    }
  }
}

int sort_values(ddcsvd_context* ctx, int N, const double* in, double* out, const VecLayout* L, Arena& a) {
  int* rank = a.take<int>(N + 8);
  return rank_values(ctx, N, in, *L, rank, out);
}

void split_bidiagonal(int N, double* a, double* b, double eps, std::vector<int>& starts, int* blk_lo,
                      int* blk_hi) {
  double bmax = 0.0;
  for (int i = 0; i < N; i++) bmax = std::max(bmax, fabs(a[i]));
  for (int i = 0; i + 1 < N; i++) bmax = std::max(bmax, fabs(b[i]));
  const double tol = 4.0 * eps * bmax;
  starts.clear();
  starts.push_back(0);
  for (int i = 0; i + 1 < N; i++) {
    if (fabs(b[i]) <= tol) {
      b[i] = 0.0;
      starts.push_back(i + 1);
    }
  }
  if (N >= 1) b[N - 1] = 0.0;
  starts.push_back(N);
  for (size_t s = 0; s + 1 < starts.size(); s++)
    for (int i = starts[s]; i < starts[s + 1]; i++) {
      blk_lo[i] = starts[s];
      blk_hi[i] = starts[s + 1];
    }
}

int bd_vectors(ddcsvd_context* ctx, int N, long long store, const double* a, const double* b,
               const double* sigma, const VecLayout* L, double* sigma_sorted, Arena& arena, bool plan_only) {
  if (N <= 0) return DDCSVD_ERR_ARG;
  double* small = arena.take<double>(6 * (size_t)N + 8);
  unsigned long long* amax = arena.take<unsigned long long>(4);
  int* rank = arena.take<int>(N + 8);
  double* big = arena.take<double>(5 * (size_t)store);
  if (plan_only) return DDCSVD_OK;
  TwParams p;
  p.N = N;
  double* dd = small;
  double* ll = small + N;
  double* dl = small + 2 * (size_t)N;
  double* dll = small + 3 * (size_t)N;
  p.dd = dd; p.ll = ll; p.dl = dl; p.dll = dll;
  p.xinv = small + 4 * (size_t)N;
  p.yinv = small + 5 * (size_t)N;
  p.sigma = sigma;
  p.L = *L;
  p.rank = rank;
  p.a = a;
  p.b = b;
  p.Lp = big; p.Um = big + store; p.S = big + 2 * store; p.Pp = big + 3 * store; p.Z = big + 4 * store;
  ktimer_begin(ctx, KC_VECTORS);
  const int sg = std::min(ceil_div(N, 256), 4 * ctx->num_sms);
  DDC_CUDA_TRY(cudaMemsetAsync(amax, 0, sizeof(unsigned long long), ctx->stream));
  tw_absmax_kernel<<<sg, 256, 0, ctx->stream>>>(N, a, b, amax);
  tw_setup_kernel<<<sg, 256, 0, ctx->stream>>>(N, a, b, amax, dd, ll, dl, dll);
  count_launch(2);
  twisted_kernel<<<ceil_div(N, 32), 32 * kTwWarps, 0, ctx->stream>>>(p);
  count_launch();
  tw_cluster_kernel<<<std::min(ceil_div(N, kClThreads), 2 * ctx->num_sms), kClThreads, 0, ctx->stream>>>(p);
  count_launch();
  DDC_TRY(rank_values(ctx, N, sigma, p.L, rank, sigma_sorted));
  tw_finalize_kernel<<<L->ntiles, dim3(32, 8), 0, ctx->stream>>>(p);
  count_launch();
  tw_zero_outside_kernel<<<std::min(N, 16 * ctx->num_sms), 128, 0, ctx->stream>>>(N, p);
  count_launch();
  ktimer_end(ctx);
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

}  // namespace ddcsvd
