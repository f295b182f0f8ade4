// adjoint.cu -- reverse-mode derivative of the thin SVD A = U diag(s) V^T
// (m >= n, k = n) for a batch of equally sized problems, FP64 or FP32.
//
//   J = U^T gU,  K = V^T gV                                (k x k)
//   F_ij = 1 / (s_j^2 - s_i^2) for i != j, 0 on the diagonal
//   M = diag(gs) + (F o (J - J^T)) S + S (F o (K - K^T)) - J S^-1
//   gA = (U M + gU S^-1) V^T
// which equals U [diag(gs) + (F o (J - J^T)) S + S (F o (K - K^T))] V^T
// + (I - U U^T) gU S^-1 V^T.  (The reference has no derivative; this is the
// standard SVD adjoint.)  Any of gU, gs, gV may be null (zero).
//
// Four kernels per call: a batched tiled GEMM for J and K, an elementwise
// kernel for M, the batched GEMM for U M (+ gU S^-1 as its C input) and for
// (U M + gU S^-1) V^T.
#include <cudaTypedefs.h>

#include "ctx_cache.hpp"
#include "internal.hpp"

namespace ddcsvd {

// C[b] (M x N, col-major, ldc) = beta * C[b] + alpha * A[b] B[b], element
// (r, k) of A[b] at A + b*as + r*ars + k*acs, element (k, c) of B[b] at
// B + b*bs + k*brs + c*bcs.  64 x 64 tiles, 256 threads with 4 x 4 outputs
// each (rows ty + 16 a, columns tx + 16 c), K in slabs of 16.  Tile loads
// walk the operand's unit-stride index fastest, so either layout of A and B
// (the adjoint reads U, V transposed and not) is read in coalesced segments.
constexpr int kBgTile = 64, kBgK = 16;

template <typename T>
__device__ __forceinline__ void bgemm_load(T (*dst)[kBgTile + 1], const T* __restrict__ src, long long s_mn,
                                           long long s_k, int mn0, int MN, int k0, int K) {
  // dst[kk][i] = element (mn0 + i, k0 + kk); the index with stride 1 varies fastest across threads
  const bool k_fast = (s_k == 1 && s_mn != 1);
  for (int idx = threadIdx.x; idx < kBgTile * kBgK; idx += blockDim.x) {
    int i, kk;
    if (k_fast) { kk = idx % kBgK; i = idx / kBgK; }
    else { i = idx % kBgTile; kk = idx / kBgTile; }
    const int r = mn0 + i, k = k0 + kk;
    dst[kk][i] = (r < MN && k < K) ? src[r * s_mn + k * s_k] : T(0);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) bgemm_kernel(int M, int N, int K, const T* __restrict__ A, long long ars,
                                                    long long acs, long long as, const T* __restrict__ B,
                                                    long long brs, long long bcs, long long bs, T* C, int ldc,
                                                    long long cs, T alpha, T beta) {
  __shared__ T At[kBgK][kBgTile + 1];
  __shared__ T Bt[kBgK][kBgTile + 1];
  const int b = blockIdx.z;
  const int r0 = blockIdx.x * kBgTile, c0 = blockIdx.y * kBgTile;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const T* Ab = A + b * as;
  const T* Bb = B + b * bs;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[a][c] = T(0);
  for (int k0 = 0; k0 < K; k0 += kBgK) {
    bgemm_load<T>(At, Ab, ars, acs, r0, M, k0, K);
    bgemm_load<T>(Bt, Bb, bcs, brs, c0, N, k0, K);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBgK; kk++) {
      T x[4], y[4];
#pragma unroll
      for (int a = 0; a < 4; a++) {
        x[a] = At[kk][ty + 16 * a];
        y[a] = Bt[kk][tx + 16 * a];
      }
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[a][c] += x[a] * y[c];
    }
    __syncthreads();
  }
  T* Cb = C + b * cs;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int r = r0 + ty + 16 * a, cc = c0 + tx + 16 * c;
      if (r < M && cc < N) {
        T* p = Cb + r + (size_t)cc * ldc;
        *p = (beta == T(0) ? T(0) : beta * *p) + alpha * acc[a][c];
      }
    }
}

// M (k x k per problem) from J, K, s, gs; P := gU S^-1 (m x k) in the same pass.
template <typename T>
__global__ void adjoint_core_kernel(int k, int m, const T* __restrict__ J, const T* __restrict__ Kv,
                                    const T* __restrict__ s, const T* __restrict__ gs, const T* __restrict__ gU,
                                    T* Mo, T* P) {
  const int b = blockIdx.y;
  const T* Jb = J ? J + (size_t)b * k * k : nullptr;
  const T* Kb = Kv ? Kv + (size_t)b * k * k : nullptr;
  const T* sb = s + (size_t)b * k;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < k * k; idx += gridDim.x * blockDim.x) {
    const int i = idx % k, j = idx / k;
    const T si = sb[i], sj = sb[j];
    T v = T(0);
    if (i == j) {
      if (gs) v += gs[(size_t)b * k + i];
    } else {
      const T f = T(1) / ((sj - si) * (sj + si));
      if (Jb) v += f * (Jb[i + (size_t)j * k] - Jb[j + (size_t)i * k]) * sj;
      if (Kb) v += si * f * (Kb[i + (size_t)j * k] - Kb[j + (size_t)i * k]);
    }
    if (Jb) v -= Jb[i + (size_t)j * k] / sj;
    Mo[(size_t)b * k * k + idx] = v;
  }
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < m * k; idx += gridDim.x * blockDim.x) {
    const int j = idx / m;
    P[(size_t)b * m * k + idx] = gU ? gU[(size_t)b * m * k + idx] / sb[j] : T(0);
  }
}

template <typename T>
static int bgemm(ddcsvd_context* ctx, int batch, int M, int N, int K, const T* A, long long ars, long long acs,
                 long long as, const T* B, long long brs, long long bcs, long long bs, T* C, int ldc, long long cs,
                 T alpha, T beta) {
  dim3 grid(ceil_div(M, kBgTile), ceil_div(N, kBgTile), batch);
  bgemm_kernel<T><<<grid, 256, 0, ctx->stream>>>(M, N, K, A, ars, acs, as, B, brs, bcs, bs, C, ldc, cs, alpha,
                                                 beta);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}

// The four launches of one adjoint on intermediates J, Kv, Mm (k x k per
// problem) and P (m x k per problem).  Launch grids carry the batch in
// gridDim.z / gridDim.y (at most 65535), so larger batches go in chunks.
constexpr int kBatchChunk = 65535;

template <typename T>
static int adjoint_enqueue(ddcsvd_context* h, int batch, int m, int n, const T* U, const T* S, const T* V,
                           const T* gU, const T* gS, const T* gV, T* gA, T* J, T* Kv, T* Mm, T* P) {
  const int k = n;
  const long long sU = (long long)m * k, sV = (long long)n * k, sK = (long long)k * k, sA = (long long)m * n;
  for (int b0 = 0; b0 < batch; b0 += kBatchChunk) {
    const int nb = std::min(kBatchChunk, batch - b0);
    const T* Ub = U + b0 * sU;
    const T* Vb = V + b0 * sV;
    const T* Sb = S + b0 * (long long)k;
    const T* gUb = gU ? gU + b0 * sU : nullptr;
    const T* gVb = gV ? gV + b0 * sV : nullptr;
    const T* gSb = gS ? gS + b0 * (long long)k : nullptr;
    T* Jb = J + b0 * sK;
    T* Kb = Kv + b0 * sK;
    T* Mb = Mm + b0 * sK;
    T* Pb = P + b0 * sU;
    // J = U^T gU, K = V^T gV
    if (gUb) DDC_TRY(bgemm<T>(h, nb, k, k, m, Ub, m, 1, sU, gUb, 1, m, sU, Jb, k, sK, T(1), T(0)));
    if (gVb) DDC_TRY(bgemm<T>(h, nb, k, k, n, Vb, n, 1, sV, gVb, 1, n, sV, Kb, k, sK, T(1), T(0)));
    dim3 g2(std::max(1, std::min(64, ceil_div(std::max(k * k, m * k), 256))), nb);
    adjoint_core_kernel<T><<<g2, 256, 0, h->stream>>>(k, m, gUb ? Jb : nullptr, gVb ? Kb : nullptr, Sb, gSb, gUb,
                                                      Mb, Pb);
    count_launch();
    DDC_CUDA_TRY(cudaGetLastError());
    // P += U M
    DDC_TRY(bgemm<T>(h, nb, m, k, k, Ub, 1, m, sU, Mb, 1, k, sK, Pb, m, sU, T(1), T(1)));
    // gA = P V^T
    DDC_TRY(bgemm<T>(h, nb, m, n, k, Pb, 1, m, sU, Vb, n, 1, sV, gA + b0 * sA, m, sA, T(1), T(0)));
  }
  return DDCSVD_OK;
}

template <typename T>
static int svd_backward(ddcsvd_context* h, int batch, int m, int n, const T* U, const T* S, const T* V, const T* gU,
                        const T* gS, const T* gV, T* gA) {
  if (!h || batch <= 0 || m <= 0 || n <= 0 || m < n || !U || !S || !V || !gA) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  const int k = n;
  const size_t kk = (size_t)k * k * batch, mk = (size_t)m * k * batch;
  Arena plan;
  plan.take<T>(kk);
  plan.take<T>(kk);
  plan.take<T>(kk);
  plan.take<T>(mk);
  DDC_TRY(ensure_workspace(h, plan.off + 4096));
  Arena a;
  a.plan = false;
  a.base = (char*)h->ws;
  T* J = a.take<T>(kk);
  T* Kv = a.take<T>(kk);
  T* Mm = a.take<T>(kk);
  T* P = a.take<T>(mk);
  DDC_TRY(reset_status(h));
  DDC_TRY(adjoint_enqueue<T>(h, batch, m, n, U, S, V, gU, gS, gV, gA, J, Kv, Mm, P));
  return check_status(h, "svd_backward");
}

// ---------------------------------------------------------------- allocation-free variant
// Some callers cannot allocate device memory at the moment they need the
// adjoint: code running inside another framework's memory pool or a
// pre-planned fixed memory budget, a real-time loop that must not reach the
// driver's allocator (cudaMalloc can synchronise the device and fail under
// fragmentation), or a context in which only caller-owned buffers may be
// touched.  For them the FP64 adjoint has a variant whose intermediates live
// in a fixed-size array compiled into this library instead of the handle's
// workspace; it needs no handle either.
constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;  // 16 MiB, held by every GPU that loads the library
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The array's host-side name is only a stand-in: its device address is
// looked up (cudaGetSymbolAddress, with the caller's context current) the
// first time a context calls, and kept per context id.
using CtxGetCurrentFn = PFN_cuCtxGetCurrent_v4000;
using CtxGetIdFn = PFN_cuCtxGetId_v12000;
static CtxValueCache<64> g_noalloc_addr;

static int driver_fn(const char* name, void** fn) {
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !*fn) {
    cudaGetLastError();
    set_last_error("driver entry point %s unavailable", name);
    return DDCSVD_ERR_CUDA;
  }
  return DDCSVD_OK;
}

static int lookup_scratch(void** p) {
  const cudaError_t e = cudaGetSymbolAddress(p, g_noalloc_scratch);
  if (e != cudaSuccess || !*p) {
    cudaGetLastError();
    set_last_error("cudaGetSymbolAddress of the adjoint scratch failed: %s", cudaGetErrorString(e));
    return DDCSVD_ERR_CUDA;
  }
  return DDCSVD_OK;
}

static int noalloc_scratch_address(char** out) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current) DDC_TRY(driver_fn("cuCtxGetCurrent", reinterpret_cast<void**>(&get_current)));
  if (!get_id) DDC_TRY(driver_fn("cuCtxGetId", reinterpret_cast<void**>(&get_id)));
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS) {
    set_last_error("cuCtxGetCurrent failed");
    return DDCSVD_ERR_CUDA;
  }
  if (!c) {
    // no context current on this thread yet: the runtime's lookup makes the
    // current device's primary context current
    void* p = nullptr;
    DDC_TRY(lookup_scratch(&p));
    if (get_current(&c) != CUDA_SUCCESS || !c) {
      set_last_error("no CUDA context is current");
      return DDCSVD_ERR_CUDA;
    }
  }
  unsigned long long id = 0;
  if (get_id(c, &id) != CUDA_SUCCESS) {
    set_last_error("cuCtxGetId failed");
    return DDCSVD_ERR_CUDA;
  }
  void* p = nullptr;
  DDC_TRY(g_noalloc_addr.get(id, &p, lookup_scratch));
  *out = static_cast<char*>(p);
  return DDCSVD_OK;
}

// Bytes of scratch one call takes: J, K and M (k x k per problem) and
// P (m x k per problem), each region rounded up to 256 bytes.
static size_t noalloc_bytes(int batch, int m, int n) {
  const size_t kk = 8 * (size_t)n * n * batch, mk = 8 * (size_t)m * n * batch;
  return 3 * (size_t)round_up((long long)kk, 256) + (size_t)round_up((long long)mk, 256);
}

static int svd_backward_f64_noalloc(cudaStream_t stream, int batch, int m, int n, const double* U, const double* S,
                                    const double* V, const double* gU, const double* gS, const double* gV,
                                    double* gA) {
  if (batch <= 0 || m <= 0 || n <= 0 || m < n || !U || !S || !V || !gA) return DDCSVD_ERR_ARG;
  const size_t need = noalloc_bytes(batch, m, n);
  if (need > kNoAllocScratchBytes) {
    set_last_error("allocation-free adjoint needs %zu bytes of scratch; its fixed limit is %zu bytes "
                   "(3 r(8 batch n^2) + r(8 batch m n), r = round up to 256): split the batch",
                   need, kNoAllocScratchBytes);
    return DDCSVD_ERR_ARG;
  }
  char* base = nullptr;
  DDC_TRY(noalloc_scratch_address(&base));
  int dev = 0;
  DDC_CUDA_TRY(cudaGetDevice(&dev));
  const int k = n;
  const size_t kk = (size_t)k * k * batch, mk = (size_t)m * k * batch;
  Arena a;
  a.plan = false;
  a.base = base;
  double* J = a.take<double>(kk);
  double* Kv = a.take<double>(kk);
  double* Mm = a.take<double>(kk);
  double* P = a.take<double>(mk);
  ddcsvd_context ctx;  // stream only: nothing here allocates
  ctx.device = dev;
  ctx.stream = stream;
  // The array keeps the previous call's contents; J, K, M and P are fully
  // overwritten before they are read, so nothing needs clearing.  The call
  // only enqueues: kernels of the same stream run in order, and a caller
  // reads gA after synchronising the stream.
  DDC_TRY(adjoint_enqueue<double>(&ctx, batch, m, n, U, S, V, gU, gS, gV, gA, J, Kv, Mm, P));
  return DDCSVD_OK;
}
}  // namespace ddcsvd

using namespace ddcsvd;

extern "C" int ddcsvd_svd_backward_f64_noalloc(void* stream, int batch, int m, int n, const double* dU,
                                               const double* dS, const double* dV, const double* gU,
                                               const double* gS, const double* gV, double* gA) {
  return svd_backward_f64_noalloc(static_cast<cudaStream_t>(stream), batch, m, n, dU, dS, dV, gU, gS, gV, gA);
}

extern "C" int ddcsvd_svd_backward_f64_device(ddcsvd_handle_t h, int batch, int m, int n, const double* dU,
                                              const double* dS, const double* dV, const double* gU,
                                              const double* gS, const double* gV, double* gA) {
  return svd_backward<double>(h, batch, m, n, dU, dS, dV, gU, gS, gV, gA);
}

extern "C" int ddcsvd_svd_backward_f32_device(ddcsvd_handle_t h, int batch, int m, int n, const float* dU,
                                              const float* dS, const float* dV, const float* gU, const float* gS,
                                              const float* gV, float* gA) {
  return svd_backward<float>(h, batch, m, n, dU, dS, dV, gU, gS, gV, gA);
}
