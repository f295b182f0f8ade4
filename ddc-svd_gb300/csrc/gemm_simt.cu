// gemm_simt.cu -- FP32 CUDA-core GEMM with strided operands and
// deterministic split-K, plus the gemm() dispatcher that picks the back end.
//
// Used for the trailing updates and the WY back-transformation in
// DDCSVD_MODE_BLOCKED_FP32, and for the small T-factor products in every
// mode.  The tensor-core back ends (gemm_tc.cu) take over the large products
// in the TF32X3 / BF16X3 modes.
#include "internal.hpp"

namespace ddcsvd {

constexpr int BM = 128, BN = 128, BK = 16, GT = 256;

struct GemmTerm {
  const float* A;
  long long ars, acs;
  const float* B;
  long long brs, bcs;
  int K;
};

// Cs[kz] (M x N, ld M) = sum over the K-range of split kz (no alpha/beta)
// when `partial` is set; otherwise C = beta*C + alpha*acc.
template <bool A_RCONTIG, bool B_CCONTIG>
__device__ __forceinline__ void load_tiles(const GemmTerm& T, int m0, int n0, int k0, int kend,
                                           int M, int N, float (*As)[BM + 4], float (*Bs)[BN + 4]) {
  const int t = threadIdx.x;
#pragma unroll
  for (int s = 0; s < (BM * BK) / GT; s++) {
    const int idx = t + GT * s;
    int r, k;
    if (A_RCONTIG) { k = idx / BM; r = idx % BM; }
    else { r = idx / BK; k = idx % BK; }
    const int gr = m0 + r, gk = k0 + k;
    As[k][r] = (gr < M && gk < kend) ? T.A[gr * T.ars + gk * T.acs] : 0.f;
  }
#pragma unroll
  for (int s = 0; s < (BN * BK) / GT; s++) {
    const int idx = t + GT * s;
    int c, k;
    if (B_CCONTIG) { k = idx / BN; c = idx % BN; }
    else { c = idx / BK; k = idx % BK; }
    const int gc = n0 + c, gk = k0 + k;
    Bs[k][c] = (gc < N && gk < kend) ? T.B[gk * T.brs + gc * T.bcs] : 0.f;
  }
}

__device__ __forceinline__ void run_term(const GemmTerm& T, int m0, int n0, int kb, int ke, int M,
                                         int N, float (*As)[BM + 4], float (*Bs)[BN + 4],
                                         float acc[8][8]) {
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const bool arc = (T.ars == 1), bcc = (T.bcs == 1);
  for (int k0 = kb; k0 < ke; k0 += BK) {
    __syncthreads();
    if (arc && bcc) load_tiles<true, true>(T, m0, n0, k0, ke, M, N, As, Bs);
    else if (arc) load_tiles<true, false>(T, m0, n0, k0, ke, M, N, As, Bs);
    else if (bcc) load_tiles<false, true>(T, m0, n0, k0, ke, M, N, As, Bs);
    else load_tiles<false, false>(T, m0, n0, k0, ke, M, N, As, Bs);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; k++) {
      float a[8], b[8];
#pragma unroll
      for (int i = 0; i < 8; i++) a[i] = As[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 8; j++) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
  }
}

__global__ void __launch_bounds__(GT) gemm_simt_kernel(int M, int N, GemmTerm T1, GemmTerm T2,
                                                       float alpha, float beta, float* C, int ldc,
                                                       float* partial, int ksplit) {
  __shared__ __align__(16) float As[BK][BM + 4];
  __shared__ __align__(16) float Bs[BK][BN + 4];
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN, kz = blockIdx.z;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
  // split-K over the concatenated K range of both terms
  const int Ktot = T1.K + T2.K;
  const int chunk = (int)round_up(ceil_div(Ktot, ksplit), BK);
  const int kb = kz * chunk, ke = min(Ktot, kb + chunk);
  if (kb < T1.K) run_term(T1, m0, n0, kb, min(ke, T1.K), M, N, As, Bs, acc);
  if (ke > T1.K && T2.K > 0)
    run_term(T2, m0, n0, max(kb, T1.K) - T1.K, ke - T1.K, M, N, As, Bs, acc);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int r = m0 + ty + 16 * i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int c = n0 + tx + 16 * j;
      if (c >= N) continue;
      if (partial) {
        partial[(size_t)kz * M * N + r + (size_t)c * M] = acc[i][j];
      } else {
        float* cp = C + r + (size_t)c * ldc;
        *cp = (beta == 0.f ? 0.f : beta * *cp) + alpha * acc[i][j];
      }
    }
  }
}

__global__ void splitk_reduce_kernel(int M, int N, int ksplit, const float* partial, float alpha,
                                     float beta, float* C, int ldc) {
  const size_t tot = (size_t)M * N;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot;
       idx += (size_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < ksplit; z++) s += partial[(size_t)z * tot + idx];
    const int r = (int)(idx % M), c = (int)(idx / M);
    float* cp = C + r + (size_t)c * ldc;
    *cp = (beta == 0.f ? 0.f : beta * *cp) + alpha * s;
  }
}

int gemm_tc(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K1, Mat A1, Mat B1, int K2,
            Mat A2, Mat B2, float alpha, float beta, float* C, int ldc, Arena* scratch);

// Transposed variant: element (r, c) of the sum goes to C[c + r * ldc].  A
// 32 x 32 tile is summed with loads along r and stored along c.
__global__ void splitk_reduce_t_kernel(int M, int N, int ksplit, const float* __restrict__ partial, float alpha,
                                       float beta, float* C, int ldc) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const size_t tot = (size_t)M * N;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + threadIdx.x, c = c0 + k;
    float s = 0.f;
    if (r < M && c < N)
      for (int z = 0; z < ksplit; z++) s += partial[(size_t)z * tot + r + (size_t)c * M];
    tile[k][threadIdx.x] = s;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    if (r < M && c < N) {
      float* cp = C + c + (size_t)r * ldc;
      *cp = (beta == 0.f ? 0.f : beta * *cp) + alpha * tile[threadIdx.x][k];
    }
  }
}

void splitk_reduce(ddcsvd_context* ctx, int M, int N, int ksplit, const float* partial, float alpha,
                   float beta, float* C, int ldc, bool trans) {
  if (trans) {
    splitk_reduce_t_kernel<<<dim3(ceil_div(M, 32), ceil_div(N, 32)), dim3(32, 8), 0, ctx->stream>>>(
        M, N, ksplit, partial, alpha, beta, C, ldc);
    count_launch();
    return;
  }
  const int blocks = std::min(4 * ctx->num_sms, ceil_div(M * N, 256));
  splitk_reduce_kernel<<<blocks, 256, 0, ctx->stream>>>(M, N, ksplit, partial, alpha, beta, C, ldc);
  count_launch();
}

// out[r * ldo + k] = k < K1 ? P1[r + k*ld1] : P2[r + (k-K1)*ld2]  (column blocks -> K-major rows)
__global__ void pack_kmajor_kernel(int rows, int K1, const float* __restrict__ P1, int ld1, int K2,
                                   const float* __restrict__ P2, int ld2, float* out, int ldo) {
  __shared__ float tile[64][33];
  const int r0 = blockIdx.x * 32;
  const int K = K1 + K2;
  for (int kb = 0; kb < K; kb += 64) {
    const int kc = min(64, K - kb);
    for (int idx = threadIdx.x; idx < kc * 32; idx += blockDim.x) {
      const int kk = idx / 32, rr = idx % 32, r = r0 + rr, k = kb + kk;
      float v = 0.f;
      if (r < rows) v = (k < K1) ? P1[r + (size_t)k * ld1] : P2[r + (size_t)(k - K1) * ld2];
      tile[kk][rr] = v;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < kc * 32; idx += blockDim.x) {
      const int rr = idx / kc, kk = idx % kc, r = r0 + rr;
      if (r < rows) out[(size_t)r * ldo + kb + kk] = tile[kk][rr];
    }
    __syncthreads();
  }
}

int pack_kmajor(ddcsvd_context* ctx, int rows, int K1, const float* P1, int ld1, int K2, const float* P2, int ld2,
                float* out, int ldo) {
  if (rows <= 0) return DDCSVD_OK;
  pack_kmajor_kernel<<<ceil_div(rows, 32), 256, 0, ctx->stream>>>(rows, K1, P1, ld1, K2, P2, ld2, out, ldo);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  return DDCSVD_OK;
}
size_t gemm_tc_scratch_bytes(GemmKind kind, int M, int N, int K);

// Split-K partial buffers: K is split only when the output has fewer tiles
// than SMs, into at most 16 and at most 2 * SMs / tiles pieces, so
// ksplit * M * N <= 2 * SMs * 128 * 128 (bounded here for up to 256 SMs).
size_t gemm_scratch_bytes(GemmKind kind, int M, int N, int K) {
  const size_t cap = (size_t)2 * 256 * 128 * 128;
  size_t simt = std::min((size_t)16 * M * N, cap) * sizeof(float) + 4096;
  if (kind == GEMM_SIMT) return simt;
  return std::max(simt, gemm_tc_scratch_bytes(kind, M, N, K));
}

int gemm_simt(ddcsvd_context* ctx, int M, int N, int K1, Mat A1, Mat B1, int K2, Mat A2, Mat B2,
              float alpha, float beta, float* C, int ldc, Arena* scratch) {
  if (M <= 0 || N <= 0) return DDCSVD_OK;
  GemmTerm T1{A1.p, A1.rs, A1.cs, B1.p, B1.rs, B1.cs, K1};
  GemmTerm T2{A2.p, A2.rs, A2.cs, B2.p, B2.rs, B2.cs, A2.p ? K2 : 0};
  const int tiles = ceil_div(M, BM) * ceil_div(N, BN);
  const int Ktot = T1.K + T2.K;
  int ksplit = 1;
  if (scratch && !scratch->plan && tiles < ctx->num_sms && Ktot >= 4 * BK * 8) {
    ksplit = std::min(std::max(1, ctx->tune[TK_SPLITK_MAX]), std::max(1, (2 * ctx->num_sms) / tiles));
    ksplit = std::min(ksplit, std::max(1, Ktot / (8 * BK)));
    while (ksplit > 1 && (size_t)ksplit * M * N * sizeof(float) > scratch->cap) ksplit--;
  }
  float* partial = (ksplit > 1) ? reinterpret_cast<float*>(scratch->base) : nullptr;
  dim3 grid(ceil_div(M, BM), ceil_div(N, BN), ksplit);
  gemm_simt_kernel<<<grid, GT, 0, ctx->stream>>>(M, N, T1, T2, alpha, beta, C, ldc, partial, ksplit);
  count_launch();
  DDC_CUDA_TRY(cudaGetLastError());
  if (ksplit > 1) {
    const int blocks = std::min(4 * ctx->num_sms, ceil_div(M * N, 256));
    splitk_reduce_kernel<<<blocks, 256, 0, ctx->stream>>>(M, N, ksplit, partial, alpha, beta, C, ldc);
    count_launch();
    DDC_CUDA_TRY(cudaGetLastError());
  }
  return DDCSVD_OK;
}

int gemm(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K1, Mat A1, Mat B1, int K2, Mat A2,
         Mat B2, float alpha, float beta, float* C, int ldc, Arena* scratch) {
  // a tensor-core kind never degrades to the CUDA-core kernel: gemm_tc fails
  // loudly when the tcgen05 path is unavailable
  if (kind != GEMM_SIMT) return gemm_tc(ctx, kind, M, N, K1, A1, B1, K2, A2, B2, alpha, beta, C, ldc, scratch);
  return gemm_simt(ctx, M, N, K1, A1, B1, K2, A2, B2, alpha, beta, C, ldc, scratch);
}

}  // namespace ddcsvd
