// dc.cu -- stage 2: double divide-and-conquer singular values (FP64).
//
// Replaces GetSingularValues_Parallel / DivideAndConquer_Parallel
// (Calculations-Parallel.c:706-874).  The recursion tree is the reference's:
// an N x (N+1) upper bidiagonal node splits at K = N/2 into a K x (K+1) and an
// (N-K-1) x (N-K) child (:731-750); leaves have N <= 2 (:722-726).  A merge
// forms z from the children's last/first right-vector rows and the rotation
// (r0, c0, s0) of their null vectors (:769-782), solves the secular equation
// for the new singular values (:48-348) and, unless it is the root,
// recomputes z-hat (Gu-Eisenstat) and the first/last rows of the merged right
// vectors for its parent (:351-588), then normalises them with phi/psi
// (:807-845).
//
// GB300 layout: one cooperative persistent kernel walks the tree bottom-up,
// one depth at a time, with five bounded grid barriers per depth:
//   P1  leaves (thread each) and merge set-up (CTA per node): parallel merge
//       of the children's sorted values, deflation, compaction;
//   P2  secular roots, one warp per root, lanes split the O(N) sums;
//   P3  z-hat, one warp per component, lanes split the O(N) product;
//   P4  merged first/last rows, one warp per root;
//   P5  merge of roots and deflated values into ascending order, row
//       normalisation (CTA per node).
// Nodes of one depth own disjoint slot ranges, so every per-node array is
// indexed by slot and lives in one N-element buffer; outputs ping-pong
// between two buffers by depth parity.
//
// Deliberate differences from the reference (shared with the FP64 oracle):
// roots are iterated to full FP64 accuracy with a two-pole rational model
// (middle way) inside a bisection bracket, differences d_j^2 - sigma_i^2 are
// formed from the nearer pole without cancellation, z-hat uses products
// instead of logs, sign(z-hat_j) = sign(z_j), tiny z_j and equal d_j deflate,
// and every iteration is capped.
#include <algorithm>
#include <vector>

#include "internal.hpp"

namespace ddcsvd {

constexpr int kDcThreads = 512;

struct DcParams {
  int N, nnodes, maxdepth, P;
  int maxit;  // FP64 iterations per secular root (the handle's limit, 80 by default)
  const int* nd_r0;
  const int* nd_nn;
  const int* nd_slot;
  const int* nd_K;
  const int* nd_c1;
  const int* nd_c2;
  const int* depth_start;  // [maxdepth + 2]
  const int* depth_merge;  // merge-node ids sorted by depth then slot
  const int* dm_start;     // [maxdepth + 2] ranges into depth_merge
  const int* dgroup;       // [maxdepth + 2] lanes per root at each depth (1..32)
  const double* b1;
  const double* b2;
  double* sig[2];
  double* F[2];
  double* L[2];
  double *ds, *zs, *hfs, *hls;
  double *dq, *zq, *fq, *lq;
  float *dqf, *zqf;  // FP32 copies of dq, zq for the first phase of the root solver
  double *dd, *fd, *ld;  // deflated entries (ascending d)
  double *tau, *zh, *rS, *rF, *rL;
  int* org;
  int* defl;
  int* nq;
  double *zz, *phi, *psi;
  double* out;
  GridBarrier* bar;
  DevStatus* st;
};

// ---------------------------------------------------------------- leaves
__device__ void dc_leaf(int nn, const double* b1, const double* b2, double* sig, double* fr,
                        double* lr, double* phi, double* psi) {
  if (nn == 1) {
    double s = hypot(b1[0], b2[0]);
    sig[0] = s;
    if (s > 0.0) {
      fr[0] = b1[0] / s; lr[0] = b2[0] / s; *phi = b2[0] / s; *psi = -b1[0] / s;
    } else {
      fr[0] = 1.0; lr[0] = 0.0; *phi = 0.0; *psi = 1.0;
    }
    return;
  }
  const double x1 = b1[0], x2 = b2[0], x3 = b1[1], x4 = b2[1];
  const double a = x1 * x1 + x2 * x2, e = x3 * x3 + x4 * x4, c = x2 * x3;
  const double det = x1 * x1 * x3 * x3 + x1 * x1 * x4 * x4 + x2 * x2 * x4 * x4;
  const double rad = hypot(0.5 * (a - e), c);
  const double lmax = 0.5 * (a + e) + rad;
  const double lmin = (lmax > 0.0) ? det / lmax : 0.0;
  const double lam[2] = {lmin, lmax};
  for (int k = 0; k < 2; k++) {
    sig[k] = sqrt(lam[k]);
    double u1a = c, u2a = lam[k] - a, u1b = lam[k] - e, u2b = c;
    double na = hypot(u1a, u2a), nb = hypot(u1b, u2b), u1, u2;
    if (na >= nb && na > 0.0) { u1 = u1a / na; u2 = u2a / na; }
    else if (nb > 0.0) { u1 = u1b / nb; u2 = u2b / nb; }
    else { u1 = (k == 0) ? 0.0 : 1.0; u2 = (k == 0) ? 1.0 : 0.0; }
    double v1 = x1 * u1, v2 = x2 * u1 + x3 * u2, v3 = x4 * u2;
    double nv = sqrt(v1 * v1 + v2 * v2 + v3 * v3);
    if (nv > 0.0) { fr[k] = v1 / nv; lr[k] = v3 / nv; }
    else { fr[k] = (k == 0) ? 1.0 : 0.0; lr[k] = 0.0; }
  }
  double n1 = x2 * x4, n2 = -x1 * x4, n3 = x1 * x3;
  double nn3 = sqrt(n1 * n1 + n2 * n2 + n3 * n3);
  if (nn3 > 0.0) { *phi = n1 / nn3; *psi = n3 / nn3; }
  else { *phi = 0.0; *psi = 1.0; }
}

// ---------------------------------------------------------------- block helpers
// Exclusive scan of per-thread counts; returns this thread's offset, total in *tot.
__device__ int block_exscan(int v, int* sh, int* tot) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    for (int w = 0; w < nw; w++) { int s = sh[w]; sh[w] = acc; acc += s; }
    sh[nw] = acc;
  }
  __syncthreads();
  int r = sh[wid] + x - v;
  *tot = sh[nw];
  __syncthreads();
  return r;
}

__device__ double block_max(double v, double* sh) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < nw; w++) r = fmax(r, sh[w]);
  __syncthreads();
  return r;
}

__device__ double block_sumd(double v, double* sh) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < nw; w++) r += sh[w];
  __syncthreads();
  return r;
}

// Cooperation policies for the per-node phases: a whole CTA for large nodes,
// one warp for nodes of at most kWarpNode entries (a batch forest has
// thousands of those per depth; a CTA each would mostly wait at barriers).
constexpr int kWarpNode = 64;
struct CtaGroup {
  int* shi;
  double* shd;
  __device__ int rank() const { return threadIdx.x; }
  __device__ int size() const { return blockDim.x; }
  __device__ void sync() const { __syncthreads(); }
  __device__ double max(double v) const { return block_max(v, shd); }
  __device__ double sum(double v) const { return block_sumd(v, shd); }
  __device__ int exscan(int v, int* tot) const { return block_exscan(v, shi, tot); }
  __device__ int any(int v) const { return __syncthreads_or(v); }
};
struct WarpGroup {
  __device__ int rank() const { return threadIdx.x & 31; }
  __device__ int size() const { return 32; }
  __device__ void sync() const { __syncwarp(); }
  __device__ double max(double v) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
  }
  __device__ double sum(double v) const { return warp_sum(v); }
  __device__ int exscan(int v, int* tot) const {
    const int lane = threadIdx.x & 31;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    *tot = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
  }
  __device__ int any(int v) const { return __any_sync(0xffffffffu, v); }
};

// number of a[0..n) < v (strict) or <= v
__device__ __forceinline__ int count_lt(const double* a, int n, double v) {
  int lo = 0, hi = n;
  while (lo < hi) { int mid = (lo + hi) >> 1; if (a[mid] < v) lo = mid + 1; else hi = mid; }
  return lo;
}
__device__ __forceinline__ int count_le(const double* a, int n, double v) {
  int lo = 0, hi = n;
  while (lo < hi) { int mid = (lo + hi) >> 1; if (a[mid] <= v) lo = mid + 1; else hi = mid; }
  return lo;
}

// ---------------------------------------------------------------- P1 merge set-up
template <class Grp>
__device__ void dc_setup_node(const DcParams& p, int node, int par, const Grp& grp) {
  const int t = grp.rank(), nt = grp.size();
  const int nn = p.nd_nn[node], slot = p.nd_slot[node], K = p.nd_K[node], r0 = p.nd_r0[node];
  const int c1 = p.nd_c1[node], c2 = p.nd_c2[node];
  const int n1 = K, n2 = nn - K - 1;
  const int cp = par ^ 1;
  const double* s1 = p.sig[cp] + slot + 1;
  const double* f1 = p.F[cp] + slot + 1;
  const double* l1 = p.L[cp] + slot + 1;
  const double* s2 = p.sig[cp] + slot + K + 1;
  const double* f2 = p.F[cp] + slot + K + 1;
  const double* l2 = p.L[cp] + slot + K + 1;
  const double bk1 = p.b1[r0 + K], bk2 = p.b2[r0 + K];
  const double phi1 = p.phi[c1], psi1 = p.psi[c1], phi2 = p.phi[c2], psi2 = p.psi[c2];
  const double r = hypot(bk1 * psi1, bk2 * phi2);  // Calculations-Parallel.c:769-771
  const double c0 = (r > 0.0) ? bk1 * psi1 / r : 1.0;
  const double s0 = (r > 0.0) ? bk2 * phi2 / r : 0.0;
  double* ds = p.ds + slot;
  double* zs = p.zs + slot;
  double* hfs = p.hfs + slot;
  double* hls = p.hls + slot;
  // parallel merge of [0] ++ child1 ++ child2 by value (ties: entry 0, then child1)
  double dmax = 0.0, zmax = 0.0;
  if (t == 0) {
    ds[0] = 0.0; zs[0] = r; hfs[0] = c0 * phi1; hls[0] = s0 * psi2;
    zmax = fabs(r);
  }
  for (int k = t; k < n1; k += nt) {
    const double v = s1[k];
    const int pos = 1 + k + count_lt(s2, n2, v);
    const double z = bk1 * l1[k];
    ds[pos] = v; zs[pos] = z; hfs[pos] = f1[k]; hls[pos] = 0.0;
    dmax = fmax(dmax, fabs(v)); zmax = fmax(zmax, fabs(z));
  }
  for (int k = t; k < n2; k += nt) {
    const double v = s2[k];
    const int pos = 1 + k + count_le(s1, n1, v);
    const double z = bk2 * f2[k];
    ds[pos] = v; zs[pos] = z; hfs[pos] = 0.0; hls[pos] = l2[k];
    dmax = fmax(dmax, fabs(v)); zmax = fmax(zmax, fabs(z));
  }
  dmax = grp.max(dmax);
  zmax = grp.max(zmax);
  const double tol = 8.0 * DBL_EPSILON * fmax(dmax, zmax);
  grp.sync();
  // deflation 1: negligible z
  const int per = ceil_div(nn, nt);
  const int lo = min(nn, t * per), hi = min(nn, lo + per);
  int cnt = 0;
  for (int k = lo; k < hi; k++) {
    int dfl = fabs(zs[k]) <= tol;
    p.defl[slot + k] = dfl;
    cnt += !dfl;
  }
  int tot;
  int off = grp.exscan(cnt, &tot);
  // positions of non-deflated entries -> compacted arrays (tentative)
  for (int k = lo; k < hi; k++)
    if (!p.defl[slot + k]) { p.dq[slot + off] = ds[k]; off++; }
  grp.sync();
  // deflation 2 needed?  (adjacent non-deflated values within tol)
  int close = 0;
  for (int k = 1 + t; k < tot; k += nt)
    if (p.dq[slot + k] - p.dq[slot + k - 1] <= tol) close = 1;
  const int need2 = grp.any(close);
  if (need2 && t == 0) {
    int prev = -1;
    for (int k = 0; k < nn; k++) {
      if (p.defl[slot + k]) continue;
      if (prev >= 0 && ds[k] - ds[prev] <= tol) {
        double rr = hypot(zs[prev], zs[k]);
        double c = zs[k] / rr, s = zs[prev] / rr;
        zs[k] = rr; zs[prev] = 0.0; p.defl[slot + prev] = 1;
        double fa = hfs[prev], fb = hfs[k], la = hls[prev], lb = hls[k];
        hfs[prev] = c * fa - s * fb; hfs[k] = s * fa + c * fb;
        hls[prev] = c * la - s * lb; hls[k] = s * la + c * lb;
      }
      prev = k;
    }
  }
  grp.sync();
  // final compaction: non-deflated -> dq/zq/fq/lq, deflated -> dd/fd/ld
  cnt = 0;
  for (int k = lo; k < hi; k++) cnt += !p.defl[slot + k];
  off = grp.exscan(cnt, &tot);
  int doff = lo - off;  // deflated entries before this thread's range
  double zzl = 0.0;
  for (int k = lo; k < hi; k++) {
    if (!p.defl[slot + k]) {
      p.dq[slot + off] = ds[k]; p.zq[slot + off] = zs[k];
      p.dqf[slot + off] = (float)ds[k]; p.zqf[slot + off] = (float)zs[k];
      p.fq[slot + off] = hfs[k]; p.lq[slot + off] = hls[k];
      zzl += zs[k] * zs[k];
      off++;
    } else {
      p.dd[slot + doff] = ds[k]; p.fd[slot + doff] = hfs[k]; p.ld[slot + doff] = hls[k];
      doff++;
    }
  }
  double zz = grp.sum(zzl);
  if (t == 0) {
    p.nq[node] = tot;
    p.zz[node] = zz;
    p.phi[node] = -s0 * phi1;  // Calculations-Parallel.c:807-808 (normalised in P5)
    p.psi[node] = c0 * psi2;
  }
}

// ---------------------------------------------------------------- lane groups
// The per-root phases run one group of G lanes (G = 1, 2, ..., 32, chosen per
// depth from its largest node) per root: small nodes of a batch forest would
// otherwise leave most of a warp idle and pay five shuffle rounds per sum.
struct LaneGroup {
  int G;          // lanes per group
  int lg;         // lane within the group
  unsigned mask;  // lanes of this group within the warp
};
__device__ __forceinline__ LaneGroup make_group(int G, int lane) {
  LaneGroup g;
  g.G = G;
  g.lg = lane & (G - 1);
  g.mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  return g;
}
template <typename T>
__device__ __forceinline__ T gsum(T v, const LaneGroup& g) {
  for (int o = g.G >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(g.mask, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T gprod(T v, const LaneGroup& g) {
  for (int o = g.G >> 1; o > 0; o >>= 1) v *= __shfl_xor_sync(g.mask, v, o);
  return v;
}

// ---------------------------------------------------------------- secular roots
__device__ __forceinline__ void sec_eval(int q, const double* d, const double* z, double dorg,
                                         double tau, int split, const LaneGroup& g, double& f, double& psi,
                                         double& dpsi, double& phi, double& dphi) {
  double ps = 0.0, dps = 0.0, ph = 0.0, dph = 0.0;
  for (int j = g.lg; j < q; j += g.G) {
    const double dj = d[j];
    const double del = (dj - dorg) * (dj + dorg) - tau;
    const double tt = z[j] / del;
    if (j <= split) { ps += z[j] * tt; dps += tt * tt; }
    else { ph += z[j] * tt; dph += tt * tt; }
  }
  psi = gsum(ps, g); dpsi = gsum(dps, g); phi = gsum(ph, g); dphi = gsum(dph, g);
  f = 1.0 + psi + phi;
}

// FP32 twin of sec_eval on the FP32 copies of d and z.
__device__ __forceinline__ void sec_eval32(int q, const float* d, const float* z, float dorg, float tau, int split,
                                           const LaneGroup& g, float& f, float& psi, float& dpsi, float& phi,
                                           float& dphi) {
  float ps = 0.f, dps = 0.f, ph = 0.f, dph = 0.f;
  for (int j = g.lg; j < q; j += g.G) {
    const float dj = d[j];
    const float del = (dj - dorg) * (dj + dorg) - tau;
    const float tt = z[j] / del;
    if (j <= split) { ps += z[j] * tt; dps += tt * tt; }
    else { ph += z[j] * tt; dph += tt * tt; }
  }
  psi = gsum(ps, g); dpsi = gsum(dps, g); phi = gsum(ph, g); dphi = gsum(dph, g);
  f = 1.f + psi + phi;
}

// One safeguarded step of the root iteration (two-pole rational model for an
// interior root, one pole for the last root), shared by the FP32 and FP64
// phases.  Returns true when converged.
template <typename T>
__device__ __forceinline__ bool sec_step(bool last, T f, T psi, T dpsi, T phi, T dphi, T da0, T db0, T eps,
                                         T& lo, T& hi, T& tau) {
  const T err = last ? T(8) * (T(1) + fabs(psi)) + fabs(tau) * dpsi
                     : T(8) * (T(1) + fabs(psi) + fabs(phi)) + fabs(tau) * (dpsi + dphi);
  if (fabs(f) <= eps * err) return true;
  if (f < T(0)) lo = tau; else hi = tau;
  if (hi - lo <= T(4) * eps * fmax(fabs(lo), fabs(hi))) return true;
  T tn;
  if (last) {
    const T da = -tau;
    const T s1 = da * da * dpsi;
    const T c = f - s1 / da;
    tn = (c != T(0)) ? tau + da + s1 / c : T(0.5) * (lo + hi);
  } else {
    const T da = da0 - tau, db = db0 - tau;
    const T s1 = da * da * dpsi, s2 = db * db * dphi;
    const T c = f - s1 / da - s2 / db;
    const T aq = c, bq = c * (da + db) + s1 + s2, cq = da * db * f;
    const T disc = sqrt(fabs(bq * bq - T(4) * aq * cq));
    T eta;
    if (aq == T(0)) eta = cq / bq;
    else if (bq <= T(0)) eta = (bq - disc) / (T(2) * aq);
    else eta = T(2) * cq / (bq + disc);
    tn = tau + eta;
  }
  if (!(tn > lo && tn < hi)) tn = T(0.5) * (lo + hi);
  tau = tn;
  return false;
}

// Root i of the node's secular equation; returns origin (local index) and tau.
// Phase 1 iterates in FP32 (GB300's FP64 pipe is narrow and these sums are
// the D&C's dominant cost) to about single precision; phase 2 continues in
// FP64 from that point inside the FP64 bracket, typically for 1-3 steps, to
// full accuracy.  A poor FP32 start (clustered poles, range trouble) only
// costs more FP64 steps: the FP64 phase keeps its own bisection safeguard.
#ifdef DDCSVD_PHASE_TRACE
__device__ unsigned g_dc_iters[64 * 84];  // [depth][FP64 iterations 0..80, 81: FP32 phase gave up early]
#endif

// f at the midpoint of (d_i, d_i+1) on the FP32 copies, with a bound on its
// error: the copies carry relative error eps32, so the difference
// del_j = (d_j - d_o)(d_j + d_o) - tau is off by about
// 3 eps32 ((|d_j| + |d_o|)^2 + |tau|); term j is off by its size times that
// over |del_j| (plus a few roundings), and the sum by q eps32 of the total.
// A term whose del_j may change sign, or lies near the FP32 subnormal range
// (where the copies lose relative precision), makes the bound infinite.
__device__ __forceinline__ void sec_mid32(int q, const float* d, const float* z, float dorg, float tau,
                                          const LaneGroup& g, float& f, float& err) {
  constexpr float e32 = FLT_EPSILON;
  float s = 0.f, sa = 0.f, ea = 0.f;
  for (int j = g.lg; j < q; j += g.G) {
    const float dj = d[j];
    const float del = (dj - dorg) * (dj + dorg) - tau;
    const float tt = z[j] * z[j] / del;
    const float ad = fabsf(dj) + fabsf(dorg);
    const float ed = 3.f * e32 * (ad * ad + fabsf(tau));
    const float at = fabsf(tt);
    s += tt;
    sa += at;
    ea += (ed < 0.5f * fabsf(del) && fabsf(del) >= 0x1p-100f) ? at * (2.f * ed / fabsf(del) + 4.f * e32) : INFINITY;
  }
  s = gsum(s, g);
  sa = gsum(sa, g);
  ea = gsum(ea, g);
  f = 1.f + s;
  err = ea + (float)(q + 2) * e32 * (1.f + sa);
}

__device__ bool sec_root(int q, const double* d, const double* z, const float* df, const float* zf, double zz,
                         int i, const LaneGroup& g, int maxit, int* origin, double* tau_out, int* iters = nullptr) {
  double f, psi, dpsi, phi, dphi;
  const bool last = (i == q - 1);
  int o;
  double lo, hi, tau, da0 = 0.0, db0 = 0.0;
  if (!last) {
    const double dd = (d[i + 1] - d[i]) * (d[i + 1] + d[i]);
    // origin = nearer pole, from the sign of f at the midpoint: from the FP32
    // copies when f clears twice its error bound, else in FP64 (an FP32 sign
    // taken without the bound picked the wrong half on close poles of a
    // batch forest, and the root then lies outside the bracket)
    float f32, e32;
    sec_mid32(q, df, zf, df[i], (float)(0.5 * dd), g, f32, e32);
    if (fabsf(f32) > 2.f * e32 && fabsf(f32) < INFINITY) {
      o = (f32 >= 0.f) ? i : i + 1;
    } else {
      sec_eval(q, d, z, d[i], 0.5 * dd, i, g, f, psi, dpsi, phi, dphi);
      o = (f >= 0.0) ? i : i + 1;
    }
    const double dorg = d[o];
    if (o == i) { lo = 0.0; hi = 0.5 * dd; tau = 0.5 * dd; }
    else { lo = -0.5 * dd; hi = 0.0; tau = -0.5 * dd; }
    da0 = (d[i] - dorg) * (d[i] + dorg);
    db0 = (d[i + 1] - dorg) * (d[i + 1] + dorg);
  } else {
    o = q - 1;
    lo = 0.0; hi = zz; tau = 0.5 * zz;
  }
  const double dorg = d[o];
  const int split = last ? q - 1 : i;
  // ---- phase 1: FP32
  {
    float lo32 = (float)lo, hi32 = (float)hi, t32 = (float)tau;
    const float d32 = df[o], da32 = (float)da0, db32 = (float)db0;
    for (int it = 0; it < 40; it++) {
      float f3, ps3, dps3, ph3, dph3;
      sec_eval32(q, df, zf, d32, t32, split, g, f3, ps3, dps3, ph3, dph3);
      if (!(fabsf(f3) < INFINITY) || !(dps3 < INFINITY) || !(dph3 < INFINITY)) break;
      if (sec_step<float>(last, f3, ps3, dps3, ph3, dph3, da32, db32, 4.f * FLT_EPSILON, lo32, hi32, t32)) break;
    }
    const double t = (double)t32;
    if (t > lo && t < hi) tau = t;
  }
  // ---- phase 2: FP64.  A step below 1e-10 |tau| is accepted without another
  // evaluation: the rational model converges at least quadratically, so the
  // remaining error is far below FP64 resolution.
  bool conv = false;
  int it = 0;
  for (; it < maxit; it++) {
    sec_eval(q, d, z, dorg, tau, split, g, f, psi, dpsi, phi, dphi);
    const double prev = tau;
    if (sec_step<double>(last, f, psi, dpsi, phi, dphi, da0, db0, DBL_EPSILON, lo, hi, tau)) {
      conv = true;
      break;
    }
    if (fabs(tau - prev) <= 1e-10 * fabs(tau)) {
      conv = true;
      break;
    }
  }
  if (iters) *iters = it;
  *origin = o;
  *tau_out = tau;
  return conv;
}

// merge node at depth d containing slot position pos (or -1)
__device__ __forceinline__ int find_node(const DcParams& p, int d, int pos) {
  int lo = p.dm_start[d], hi = p.dm_start[d + 1];
  // largest merge node with slot <= pos
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (p.nd_slot[p.depth_merge[mid]] <= pos) lo = mid + 1; else hi = mid;
  }
  if (lo == p.dm_start[d]) return -1;
  int node = p.depth_merge[lo - 1];
  int slot = p.nd_slot[node];
  return (pos < slot + p.nd_nn[node]) ? node : -1;
}

// ---------------------------------------------------------------- P5 final merge
template <class Grp>
__device__ void dc_finish_node(const DcParams& p, int node, int par, bool rows, const Grp& grp) {
  const int t = grp.rank(), nt = grp.size();
  const int nn = p.nd_nn[node], slot = p.nd_slot[node];
  const int q = p.nq[node], nd = nn - q;
  const double* rs = p.rS + slot;
  const double* dd = p.dd + slot;
  double* sig = p.sig[par] + slot;
  double* F = p.F[par] + slot;
  double* L = p.L[par] + slot;
  for (int k = t; k < q; k += nt) {
    const int pos = k + count_lt(dd, nd, rs[k]);
    sig[pos] = rs[k];
    if (rows) { F[pos] = p.rF[slot + k]; L[pos] = p.rL[slot + k]; }
  }
  for (int k = t; k < nd; k += nt) {
    const int pos = k + count_le(rs, q, dd[k]);
    sig[pos] = dd[k];
    if (rows) { F[pos] = p.fd[slot + k]; L[pos] = p.ld[slot + k]; }
  }
  if (!rows) return;
  grp.sync();
  double sf = 0.0, sl = 0.0;
  for (int k = t; k < nn; k += nt) { sf += F[k] * F[k]; sl += L[k] * L[k]; }
  sf = grp.sum(sf);
  sl = grp.sum(sl);
  const double ph = p.phi[node], ps = p.psi[node];
  const double nf = sqrt(sf + ph * ph), nl = sqrt(sl + ps * ps);
  for (int k = t; k < nn; k += nt) {
    if (nf > 0.0) F[k] /= nf;
    if (nl > 0.0) L[k] /= nl;
  }
  grp.sync();
  if (t == 0) {
    if (nf > 0.0) p.phi[node] = ph / nf;
    if (nl > 0.0) p.psi[node] = ps / nl;
  }
}

#ifdef DDCSVD_PHASE_TRACE
__device__ unsigned long long g_dc_trace[64 * 16];
#endif
// phase marks of CTA 0, one row per depth (slots: 0 start, 1 after P1, 2 after
// its barrier, 3 after P2, 4 barrier, 5 P3, 6 barrier, 7 P4, 8 barrier, 9 P5,
// 10 barrier)
#ifdef DDCSVD_PHASE_TRACE
#define DMARK(slot)                                                               \
  do {                                                                            \
    if (blockIdx.x == 0 && threadIdx.x == 0 && d < 64) g_dc_trace[d * 16 + (slot)] = global_ns(); \
  } while (0)
#else
#define DMARK(slot) \
  do {              \
  } while (0)
#endif

__global__ void __launch_bounds__(kDcThreads, 1) dc_kernel(DcParams p) {
  __shared__ int shi[40];
  __shared__ double shd[40];
  const int t = threadIdx.x, lane = t & 31;
  const int gw = (blockIdx.x * blockDim.x + t) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int gt = blockIdx.x * blockDim.x + t, nthreads = gridDim.x * blockDim.x;
  for (int d = p.maxdepth; d >= 0; d--) {
    const int par = d & 1;
    const bool rows = d > 0;
    DMARK(0);
    // ---- P1a leaves of this depth (thread each)
    for (int k = p.depth_start[d] + gt; k < p.depth_start[d + 1]; k += nthreads) {
      if (p.nd_K[k] >= 0) continue;
      const int nn = p.nd_nn[k], slot = p.nd_slot[k], r0 = p.nd_r0[k];
      double phi, psi;
      dc_leaf(nn, p.b1 + r0, p.b2 + r0, p.sig[par] + slot, p.F[par] + slot, p.L[par] + slot, &phi, &psi);
      p.phi[k] = phi;
      p.psi[k] = psi;
    }
    // ---- P1b merge set-up: CTA per large node, warp per small node
    {
      const CtaGroup cg{shi, shd};
      for (int mi = p.dm_start[d] + blockIdx.x; mi < p.dm_start[d + 1]; mi += gridDim.x)
        if (p.nd_nn[p.depth_merge[mi]] > kWarpNode) dc_setup_node(p, p.depth_merge[mi], par, cg);
      const WarpGroup wg;
      for (int mi = p.dm_start[d] + gw; mi < p.dm_start[d + 1]; mi += nwarps)
        if (p.nd_nn[p.depth_merge[mi]] <= kWarpNode) dc_setup_node(p, p.depth_merge[mi], par, wg);
    }
    if (p.dm_start[d + 1] == p.dm_start[d]) {  // only leaves at this depth
      if (d > 0 && !grid_sync(p.bar, p.P, p.st, 600 + d)) return;
      continue;
    }
    DMARK(1);
    if (!grid_sync(p.bar, p.P, p.st, 100 + d)) return;
    DMARK(2);
    // ---- P2 secular roots (lane group per root)
    const LaneGroup g = make_group(p.dgroup[d], lane);
    const int gid = gt / g.G, ngroups = nthreads / g.G;
    for (int pos = gid; pos < p.N; pos += ngroups) {
      const int node = find_node(p, d, pos);
      if (node < 0) continue;
      const int slot = p.nd_slot[node], i = pos - slot, q = p.nq[node];
      if (i >= q) continue;
      int o;
      double tau;
      int its = 0;
      bool ok = sec_root(q, p.dq + slot, p.zq + slot, p.dqf + slot, p.zqf + slot, p.zz[node], i, g, p.maxit, &o,
                         &tau, &its);
#ifdef DDCSVD_PHASE_TRACE
      if (g.lg == 0 && d < 64) atomicAdd(&g_dc_iters[d * 84 + min(its, 80)], 1u);
#else
      (void)its;
#endif
      if (g.lg == 0) {
        p.org[pos] = o;
        p.tau[pos] = tau;
        const double dorg = p.dq[slot + o];
        p.rS[pos] = sqrt(dorg * dorg + tau);
        if (!ok) set_error(p.st, DDCSVD_ERR_NOCONV, pos);
      }
    }
    DMARK(3);
    if (rows) {
      if (!grid_sync(p.bar, p.P, p.st, 200 + d)) return;
      DMARK(4);
      // ---- P3 z-hat (lane group per component)
      for (int pos = gid; pos < p.N; pos += ngroups) {
        const int node = find_node(p, d, pos);
        if (node < 0) continue;
        const int slot = p.nd_slot[node], j = pos - slot, q = p.nq[node];
        if (j >= q) continue;
        const double* dq = p.dq + slot;
        const double* tau = p.tau + slot;
        const int* org = p.org + slot;
        const double dj = dq[j];
        double prod = 1.0;
        for (int k = g.lg; k < q - 1; k += g.G) {
          const int ok = org[k];
          const double num = tau[k] - (dj - dq[ok]) * (dj + dq[ok]);
          const int kk = (k < j) ? k : k + 1;
          const double den = (dq[kk] - dj) * (dq[kk] + dj);
          prod *= num / den;
        }
        prod = gprod(prod, g);
        if (g.lg == 0) {
          const int ol = org[q - 1];
          prod *= tau[q - 1] - (dj - dq[ol]) * (dj + dq[ol]);
          const double a = sqrt(fabs(prod));
          p.zh[pos] = (p.zq[pos] >= 0.0) ? a : -a;
        }
      }
      DMARK(5);
      if (!grid_sync(p.bar, p.P, p.st, 300 + d)) return;
      DMARK(6);
      // ---- P4 rows of the merged right vectors (lane group per root)
      for (int pos = gid; pos < p.N; pos += ngroups) {
        const int node = find_node(p, d, pos);
        if (node < 0) continue;
        const int slot = p.nd_slot[node], i = pos - slot, q = p.nq[node];
        if (i >= q) continue;
        const double* dq = p.dq + slot;
        const double dorg = dq[p.org[pos]], ti = p.tau[pos];
        double nv = 0.0, sf = 0.0, sl = 0.0;
        for (int j = g.lg; j < q; j += g.G) {
          const double dj = dq[j];
          const double del = (dj - dorg) * (dj + dorg) - ti;
          const double v = p.zh[slot + j] / del;
          nv += v * v;
          sf += v * p.fq[slot + j];
          sl += v * p.lq[slot + j];
        }
        nv = gsum(nv, g); sf = gsum(sf, g); sl = gsum(sl, g);
        if (g.lg == 0) {
          nv = sqrt(nv);
          p.rF[pos] = sf / nv;
          p.rL[pos] = sl / nv;
        }
      }
    }
    DMARK(7);
    if (!grid_sync(p.bar, p.P, p.st, 400 + d)) return;
    DMARK(8);
    // ---- P5 final merge + normalisation (CTA per node)
    {
      const CtaGroup cg{shi, shd};
      for (int mi = p.dm_start[d] + blockIdx.x; mi < p.dm_start[d + 1]; mi += gridDim.x)
        if (p.nd_nn[p.depth_merge[mi]] > kWarpNode) dc_finish_node(p, p.depth_merge[mi], par, rows, cg);
      const WarpGroup wg;
      for (int mi = p.dm_start[d] + gw; mi < p.dm_start[d + 1]; mi += nwarps)
        if (p.nd_nn[p.depth_merge[mi]] <= kWarpNode) dc_finish_node(p, p.depth_merge[mi], par, rows, wg);
    }
    DMARK(9);
    if (d > 0 && !grid_sync(p.bar, p.P, p.st, 500 + d)) return;
    DMARK(10);
  }
}

// ---------------------------------------------------------------- tree per CTA
// A forest of many small trees (a batch of small bidiagonals): every CTA takes
// whole trees, largest first, from an atomic counter and runs their depths
// bottom-up with block barriers only -- the same leaf, set-up, root, z-hat,
// row and finish steps as dc_kernel, without its grid barriers (where CTAs
// waited for the slowest one at every phase of every depth).
struct DcTrees {
  int ntrees;
  const int* tree_seg;   // [ntrees + 1] ranges of segments
  const int* seg_lo;     // [nseg + 1] ranges of `nodes` (merges, then leaves)
  const int* seg_mid;    // [nseg] end of the merges
  const int* seg_depth;  // [nseg]
  const int* seg_G;      // [nseg] lanes per root
  const int* nodes;
  const int* order;      // trees, largest first
  int* counter;
};
constexpr int kDcTreeThreads = 256;

// merge node of segment [lo, mid) containing slot position pos (or -1)
__device__ __forceinline__ int seg_find(const DcParams& p, const int* nodes, int lo, int mid, int pos) {
  int a = lo, b = mid;
  while (a < b) {
    const int c = (a + b) >> 1;
    if (p.nd_slot[nodes[c]] <= pos) a = c + 1; else b = c;
  }
  if (a == lo) return -1;
  const int node = nodes[a - 1];
  return (pos < p.nd_slot[node] + p.nd_nn[node]) ? node : -1;
}

__global__ void __launch_bounds__(kDcTreeThreads, 2) dc_tree_kernel(DcParams p, DcTrees tr) {
  __shared__ int shi[40];
  __shared__ double shd[40];
  __shared__ int s_tree;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
  while (true) {
    if (t == 0) s_tree = atomicAdd(tr.counter, 1);
    __syncthreads();
    const int qi = s_tree;
    __syncthreads();
    if (qi >= tr.ntrees) break;
    const int tree = tr.order[qi];
    for (int k = tr.tree_seg[tree]; k < tr.tree_seg[tree + 1]; k++) {
      const int lo = tr.seg_lo[k], mid = tr.seg_mid[k], hi = tr.seg_lo[k + 1];
      const int d = tr.seg_depth[k], par = d & 1;
      const bool rows = d > 0;
      // ---- leaves (thread each)
      for (int x = mid + t; x < hi; x += blockDim.x) {
        const int node = tr.nodes[x];
        const int nn = p.nd_nn[node], slot = p.nd_slot[node], r0 = p.nd_r0[node];
        double phi, psi;
        dc_leaf(nn, p.b1 + r0, p.b2 + r0, p.sig[par] + slot, p.F[par] + slot, p.L[par] + slot, &phi, &psi);
        p.phi[node] = phi;
        p.psi[node] = psi;
      }
      if (mid == lo) {  // only leaves at this depth
        __syncthreads();
        continue;
      }
      // ---- merge set-up: the CTA for large nodes, a warp for small ones
      {
        const CtaGroup cg{shi, shd};
        for (int x = lo; x < mid; x++)
          if (p.nd_nn[tr.nodes[x]] > kWarpNode) dc_setup_node(p, tr.nodes[x], par, cg);
        const WarpGroup wg;
        for (int x = lo + wid; x < mid; x += nw)
          if (p.nd_nn[tr.nodes[x]] <= kWarpNode) dc_setup_node(p, tr.nodes[x], par, wg);
      }
      __syncthreads();
      const LaneGroup g = make_group(tr.seg_G[k], lane);
      const int gid = t / g.G, ngroups = blockDim.x / g.G;
      const int pos0 = p.nd_slot[tr.nodes[lo]];
      const int pos1 = p.nd_slot[tr.nodes[mid - 1]] + p.nd_nn[tr.nodes[mid - 1]];
      // ---- secular roots (lane group per root)
      for (int pos = pos0 + gid; pos < pos1; pos += ngroups) {
        const int node = seg_find(p, tr.nodes, lo, mid, pos);
        if (node < 0) continue;
        const int slot = p.nd_slot[node], i = pos - slot, q = p.nq[node];
        if (i >= q) continue;
        int o;
        double tau;
        const bool ok =
            sec_root(q, p.dq + slot, p.zq + slot, p.dqf + slot, p.zqf + slot, p.zz[node], i, g, p.maxit, &o, &tau);
        if (g.lg == 0) {
          p.org[pos] = o;
          p.tau[pos] = tau;
          const double dorg = p.dq[slot + o];
          p.rS[pos] = sqrt(dorg * dorg + tau);
          if (!ok) set_error(p.st, DDCSVD_ERR_NOCONV, pos);
        }
      }
      __syncthreads();
      if (rows) {
        // ---- z-hat (lane group per component)
        for (int pos = pos0 + gid; pos < pos1; pos += ngroups) {
          const int node = seg_find(p, tr.nodes, lo, mid, pos);
          if (node < 0) continue;
          const int slot = p.nd_slot[node], j = pos - slot, q = p.nq[node];
          if (j >= q) continue;
          const double* dq = p.dq + slot;
          const double* tau = p.tau + slot;
          const int* org = p.org + slot;
          const double dj = dq[j];
          double prod = 1.0;
          for (int kk = g.lg; kk < q - 1; kk += g.G) {
            const int ok = org[kk];
            const double num = tau[kk] - (dj - dq[ok]) * (dj + dq[ok]);
            const int k2 = (kk < j) ? kk : kk + 1;
            const double den = (dq[k2] - dj) * (dq[k2] + dj);
            prod *= num / den;
          }
          prod = gprod(prod, g);
          if (g.lg == 0) {
            const int ol = org[q - 1];
            prod *= tau[q - 1] - (dj - dq[ol]) * (dj + dq[ol]);
            const double a = sqrt(fabs(prod));
            p.zh[pos] = (p.zq[pos] >= 0.0) ? a : -a;
          }
        }
        __syncthreads();
        // ---- rows of the merged right vectors (lane group per root)
        for (int pos = pos0 + gid; pos < pos1; pos += ngroups) {
          const int node = seg_find(p, tr.nodes, lo, mid, pos);
          if (node < 0) continue;
          const int slot = p.nd_slot[node], i = pos - slot, q = p.nq[node];
          if (i >= q) continue;
          const double* dq = p.dq + slot;
          const double dorg = dq[p.org[pos]], ti = p.tau[pos];
          double nv = 0.0, sf = 0.0, sl = 0.0;
          for (int j = g.lg; j < q; j += g.G) {
            const double dj = dq[j];
            const double del = (dj - dorg) * (dj + dorg) - ti;
            const double v = p.zh[slot + j] / del;
            nv += v * v;
            sf += v * p.fq[slot + j];
            sl += v * p.lq[slot + j];
          }
          nv = gsum(nv, g); sf = gsum(sf, g); sl = gsum(sl, g);
          if (g.lg == 0) {
            nv = sqrt(nv);
            p.rF[pos] = sf / nv;
            p.rL[pos] = sl / nv;
          }
        }
        __syncthreads();
      }
      // ---- final merge + normalisation
      {
        const CtaGroup cg{shi, shd};
        for (int x = lo; x < mid; x++)
          if (p.nd_nn[tr.nodes[x]] > kWarpNode) dc_finish_node(p, tr.nodes[x], par, rows, cg);
        const WarpGroup wg;
        for (int x = lo + wid; x < mid; x += nw)
          if (p.nd_nn[tr.nodes[x]] <= kWarpNode) dc_finish_node(p, tr.nodes[x], par, rows, wg);
      }
      __syncthreads();
    }
  }
}

__global__ void dc_copy_out(int N, const double* s, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) out[i] = s[i];
}

// ---------------------------------------------------------------- host: forest
// One tree per unreduced block [lo, hi) of the (split) bidiagonal; a block's
// singular values occupy slots [lo, hi).  Nodes are created depth-first; a
// stable counting sort by depth then gives the order the kernel walks (by
// depth, slots ascending within a depth) without a comparison sort: a batch
// forest has ~10^5 nodes and this runs on the host between two kernels.
namespace {
struct Forest {
  std::vector<int> r0, nn, slot, K, c1, c2, depth;
  int maxdepth = 0;
  int add(int r, int n, int sl, int d) {
    const int id = (int)r0.size();
    r0.push_back(r); nn.push_back(n); slot.push_back(sl);
    K.push_back(-1); c1.push_back(-1); c2.push_back(-1); depth.push_back(d);
    if (d > maxdepth) maxdepth = d;
    return id;
  }
  int build(int r, int n, int sl, int d) {
    const int id = add(r, n, sl, d);
    if (n > 2) {
      const int k = n / 2;
      K[id] = k;
      const int a = build(r, k, sl + 1, d + 1);
      const int b = build(r + k + 1, n - k - 1, sl + k + 1, d + 1);
      c1[id] = a;
      c2[id] = b;
    }
    return id;
  }
};
}  // namespace

void dc_build_host(int N, const std::vector<int>& starts, DcHost& H, int terms_per_lane) {
  Forest T;
  const size_t cap = 2 * (size_t)N + 8;
  T.r0.reserve(cap); T.nn.reserve(cap); T.slot.reserve(cap); T.K.reserve(cap);
  T.c1.reserve(cap); T.c2.reserve(cap); T.depth.reserve(cap);
  std::vector<int> tree_of;  // creation index -> tree
  tree_of.reserve(cap);
  int ntrees = 0;
  for (size_t b = 0; b + 1 < starts.size(); b++) {
    const int lo = starts[b], hi = starts[b + 1];
    if (hi > lo) {
      T.build(lo, hi - lo, lo, 0);
      tree_of.resize(T.r0.size(), ntrees);
      ntrees++;
    }
  }
  const int nnodes = (int)T.r0.size();
  const int md = T.maxdepth;
  // stable counting sort by depth (depth-first creation keeps slots ascending within a depth)
  std::vector<int> ds(md + 2, 0);
  for (int i = 0; i < nnodes; i++) ds[T.depth[i] + 1]++;
  for (int d = 0; d <= md; d++) ds[d + 1] += ds[d];
  std::vector<int> newid(nnodes), fill(ds.begin(), ds.end() - 1);
  for (int i = 0; i < nnodes; i++) newid[i] = fill[T.depth[i]]++;
  std::vector<int> r0(nnodes), nn(nnodes), slot(nnodes), K(nnodes), c1(nnodes), c2(nnodes), dep(nnodes);
  for (int o = 0; o < nnodes; o++) {
    const int i = newid[o];
    dep[i] = T.depth[o];
    r0[i] = T.r0[o]; nn[i] = T.nn[o]; slot[i] = T.slot[o]; K[i] = T.K[o];
    c1[i] = T.c1[o] >= 0 ? newid[T.c1[o]] : -1;
    c2[i] = T.c2[o] >= 0 ? newid[T.c2[o]] : -1;
  }
  std::vector<int> dms(md + 2, 0), dmerge;
  dmerge.reserve(nnodes);
  for (int d = 0; d <= md; d++) {
    dms[d] = (int)dmerge.size();
    for (int i = ds[d]; i < ds[d + 1]; i++) if (K[i] >= 0) dmerge.push_back(i);
  }
  dms[md + 1] = (int)dmerge.size();
  // lanes per root at each depth: about terms_per_lane terms of the largest node per lane
  const int tpl = std::max(1, terms_per_lane);
  std::vector<int> dgroup(md + 2, 1);
  for (int d = 0; d <= md; d++) {
    int mx = 0;
    for (int k = dms[d]; k < dms[d + 1]; k++) mx = std::max(mx, nn[dmerge[k]]);
    int G = 1;
    while (G < 32 && G * tpl < mx) G <<= 1;
    dgroup[d] = G;
  }
  H.nnodes = nnodes;
  H.maxdepth = md;
  H.ndm = (int)dmerge.size();
  H.ints.clear();
  H.ints.reserve(6 * (size_t)nnodes + 3 * (md + 2) + dmerge.size());
  auto app = [&](const std::vector<int>& v) { H.ints.insert(H.ints.end(), v.begin(), v.end()); };
  app(r0); app(nn); app(slot); app(K); app(c1); app(c2); app(ds); app(dms); app(dmerge); app(dgroup);
  // ---- per-tree schedule: each tree's nodes by depth, deepest first; within
  // a depth its merge nodes (ascending slot) then its leaves.  New ids are
  // sorted by (depth, slot), so one ascending pass lists every tree's nodes
  // by depth already.
  // stable counting sort of the node ids by tree (keeps (depth, slot) order)
  std::vector<int> tstart(ntrees + 1, 0), bytree(nnodes);
  for (int o = 0; o < nnodes; o++) tstart[tree_of[o] + 1]++;
  for (int tr = 0; tr < ntrees; tr++) tstart[tr + 1] += tstart[tr];
  {
    std::vector<int> tree_new(nnodes), cur(tstart.begin(), tstart.end() - 1);
    for (int o = 0; o < nnodes; o++) tree_new[newid[o]] = tree_of[o];
    for (int i = 0; i < nnodes; i++) bytree[cur[tree_new[i]]++] = i;
  }
  std::vector<int> tree_seg(ntrees + 1, 0), seg_lo, seg_mid, seg_depth, seg_G, nodes_out, order(ntrees), tsize(ntrees);
  nodes_out.reserve(nnodes);
  seg_lo.reserve(nnodes + 1); seg_mid.reserve(nnodes); seg_depth.reserve(nnodes); seg_G.reserve(nnodes);
  std::vector<int> bounds;  // depth-group boundaries of one tree (reused)
  for (int tr = 0; tr < ntrees; tr++) {
    const int* v = bytree.data() + tstart[tr];
    const int cnt = tstart[tr + 1] - tstart[tr];
    tsize[tr] = cnt ? nn[v[0]] : 0;  // the root (depth 0) comes first
    tree_seg[tr] = (int)seg_lo.size();
    bounds.clear();
    bounds.push_back(0);
    for (int x = 1; x < cnt; x++)
      if (dep[v[x]] != dep[v[x - 1]]) bounds.push_back(x);
    bounds.push_back(cnt);
    for (int gi = (int)bounds.size() - 2; gi >= 0; gi--) {  // deepest first
      const int a = bounds[gi], b = bounds[gi + 1];
      seg_lo.push_back((int)nodes_out.size());
      int mx = 0;
      for (int x = a; x < b; x++)
        if (K[v[x]] >= 0) {
          nodes_out.push_back(v[x]);
          mx = std::max(mx, nn[v[x]]);
        }
      seg_mid.push_back((int)nodes_out.size());
      for (int x = a; x < b; x++)
        if (K[v[x]] < 0) nodes_out.push_back(v[x]);
      seg_depth.push_back(dep[v[a]]);
      int G = 1;
      while (G < 32 && G * tpl < mx) G <<= 1;
      seg_G.push_back(G);
    }
  }
  const int nseg = (int)seg_lo.size();
  tree_seg[ntrees] = nseg;
  seg_lo.push_back((int)nodes_out.size());
  for (int tr = 0; tr < ntrees; tr++) order[tr] = tr;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return tsize[a] > tsize[b]; });
  H.ntrees = ntrees;
  H.nseg = nseg;
  H.maxtree = ntrees ? tsize[order[0]] : 0;
  H.tree_off = H.ints.size();
  app(tree_seg); app(seg_lo); app(seg_mid); app(seg_depth); app(seg_G); app(nodes_out); app(order);
}

// ints of the node table: 9 arrays of at most 2N + 8 entries, the per-depth
// tables, and the per-tree schedule (at most N trees, 2N + 8 segments and nodes)
size_t dc_max_ints(int N) { return 9 * (size_t)(2 * N + 8) + 2 * 64 + 16 + 2 * ((size_t)N + 1) + 5 * (2 * (size_t)N + 9); }


int dc_sigma(ddcsvd_context* ctx, int N, const double* b1, const double* b2, double* sigma,
             const DcHost* H, const int* dints, Arena& a, bool plan_only) {
  if (N <= 0) return DDCSVD_ERR_ARG;
  const int maxnodes = 2 * N + 8;
  int* scratch_ints = a.take<int>((size_t)N * 2 + maxnodes);
  double* dbl = a.take<double>((size_t)N * 25 + 3 * (size_t)maxnodes + 8);
  float* flt = a.take<float>((size_t)N * 2 + 8);
  GridBarrier* bar = a.take<GridBarrier>(4);
  if (plan_only) return DDCSVD_OK;
  const int nnodes = H->nnodes, md = H->maxdepth;
  DcParams p;
  p.N = N; p.nnodes = nnodes; p.maxdepth = md;
  p.maxit = ctx->sec_maxit;
  size_t o = 0;
  p.nd_r0 = dints + o; o += nnodes;
  p.nd_nn = dints + o; o += nnodes;
  p.nd_slot = dints + o; o += nnodes;
  p.nd_K = dints + o; o += nnodes;
  p.nd_c1 = dints + o; o += nnodes;
  p.nd_c2 = dints + o; o += nnodes;
  p.depth_start = dints + o; o += md + 2;
  p.dm_start = dints + o; o += md + 2;
  p.depth_merge = dints + o; o += H->ndm;
  p.dgroup = dints + o; o += md + 2;
  p.org = scratch_ints;
  p.defl = scratch_ints + N;
  p.nq = scratch_ints + 2 * (size_t)N;
  p.b1 = b1; p.b2 = b2;
  double* q = dbl;
  for (int k = 0; k < 2; k++) { p.sig[k] = q; q += N; p.F[k] = q; q += N; p.L[k] = q; q += N; }
  p.ds = q; q += N; p.zs = q; q += N; p.hfs = q; q += N; p.hls = q; q += N;
  p.dq = q; q += N; p.zq = q; q += N; p.fq = q; q += N; p.lq = q; q += N;
  p.dd = q; q += N; p.fd = q; q += N; p.ld = q; q += N;
  p.tau = q; q += N; p.zh = q; q += N; p.rS = q; q += N; p.rF = q; q += N; p.rL = q; q += N;
  p.zz = q; q += maxnodes; p.phi = q; q += maxnodes; p.psi = q; q += maxnodes;
  p.dqf = flt; p.zqf = flt + N;
  p.out = sigma;
  p.bar = bar;
  p.st = ctx->d_status;
  // a forest of many small trees: whole trees per CTA, no grid barriers
  if (H->ntrees >= 64 && H->maxtree <= 1024) {
    DcTrees tr;
    size_t q2 = H->tree_off;
    const int nt = H->ntrees, ns = H->nseg;
    tr.ntrees = nt;
    tr.tree_seg = dints + q2; q2 += nt + 1;
    tr.seg_lo = dints + q2; q2 += ns + 1;
    tr.seg_mid = dints + q2; q2 += ns;
    tr.seg_depth = dints + q2; q2 += ns;
    tr.seg_G = dints + q2; q2 += ns;
    tr.nodes = dints + q2; q2 += nnodes;
    tr.order = dints + q2;
    tr.counter = reinterpret_cast<int*>(bar);
    int occ = 0;
    DDC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dc_tree_kernel, kDcTreeThreads, 0));
    const int grid = std::max(1, std::min(nt, ctx->num_sms * std::max(occ, 1)));
    DDC_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(GridBarrier), ctx->stream));
    ktimer_begin(ctx, KC_DC);
    dc_tree_kernel<<<grid, kDcTreeThreads, 0, ctx->stream>>>(p, tr);
    ktimer_end(ctx);
    count_launch();
    dc_copy_out<<<std::min(ceil_div(N, 256), 1024), 256, 0, ctx->stream>>>(N, p.sig[0], sigma);
    count_launch();
    DDC_CUDA_TRY(cudaGetLastError());
    return DDCSVD_OK;
  }
  int occ = 0;
  DDC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, dc_kernel, kDcThreads, 0));
  if (occ < 1) {
    set_last_error("dc_kernel cannot be resident");
    return DDCSVD_ERR_CUDA;
  }
  const int P = std::min(ctx->num_sms, std::max(1, ceil_div(N, 16)));
  p.P = P;
  DDC_CUDA_TRY(cudaMemsetAsync(bar, 0, sizeof(GridBarrier), ctx->stream));
  void* argv[] = {&p};
  ktimer_begin(ctx, KC_DC);
  DDC_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)dc_kernel, dim3(P), dim3(kDcThreads), argv, 0,
                                           ctx->stream));
  ktimer_end(ctx);
  count_launch();
  dc_copy_out<<<std::min(ceil_div(N, 256), 1024), 256, 0, ctx->stream>>>(N, p.sig[0], sigma);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

}  // namespace ddcsvd

#ifdef DDCSVD_PHASE_TRACE
extern "C" int ddcsvd_dc_trace_read(unsigned long long* out) {
  return (int)cudaMemcpyFromSymbol(out, ddcsvd::g_dc_trace, sizeof(ddcsvd::g_dc_trace));
}
extern "C" int ddcsvd_dc_iters_read(unsigned* out) {
  return (int)cudaMemcpyFromSymbol(out, ddcsvd::g_dc_iters, sizeof(ddcsvd::g_dc_iters));
}
#endif
