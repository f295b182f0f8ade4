// tune.cu -- launch-configuration autotuner.
//
// The handle carries a small vector of launch knobs (TuneKnob: split-K cap
// and tile width of the GEMMs, CTA size and shared-memory residency of the
// batched stage 1, lane-group sizing of the D&C, QR first for tall matrices).  None of them changes the
// arithmetic beyond the summation order of split-K and of the D&C sums, so
// the tuner only measures time: a coordinate search that, knob by knob, runs
// the caller's shape (or batch) on seeded synthetic data for each candidate
// value, times it with CUDA events on the handle's stream and keeps the
// fastest.  The result stays in the handle (ddcsvd_get_tuning reads it back,
// ddcsvd_set_tuning restores a saved vector).
#include <string.h>

#include <vector>

#include "internal.hpp"

namespace ddcsvd {

// U[-1, 1) from a 32-bit integer hash of the index (deterministic)
__global__ void fill_uniform_kernel(float* x, size_t n, unsigned seed) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)i * 2654435761u ^ seed;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    x[i] = (float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f;
  }
}

namespace {
struct Candidates {
  int knob;
  std::vector<int> values;
};

// Runs `run` reps times per candidate value of every knob in turn; keeps the
// fastest value of each knob before moving to the next.
template <typename Run>
int coordinate_search(ddcsvd_context* h, const std::vector<Candidates>& space, int reps, Run run) {
  cudaEvent_t e0, e1;
  DDC_CUDA_TRY(cudaEventCreate(&e0));
  DDC_CUDA_TRY(cudaEventCreate(&e1));
  int rc = DDCSVD_OK;
  for (const Candidates& c : space) {
    int best = h->tune[c.knob];
    float best_ms = 1e30f;
    for (int v : c.values) {
      h->tune[c.knob] = v;
      rc = run();  // warm-up (workspace growth, first launches)
      if (rc) break;
      float ms = 1e30f;
      for (int r = 0; r < reps && rc == DDCSVD_OK; r++) {
        cudaEventRecord(e0, h->stream);
        rc = run();
        cudaEventRecord(e1, h->stream);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        ms = std::min(ms, t);
      }
      if (rc) break;
      if (ms < best_ms) {
        best_ms = ms;
        best = v;
      }
    }
    h->tune[c.knob] = best;
    if (rc) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}
}  // namespace

}  // namespace ddcsvd

using namespace ddcsvd;

extern "C" int ddcsvd_set_tuning(ddcsvd_handle_t h, const int* values, int count) {
  if (!h || !values || count < 0) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  for (int k = 0; k < std::min(count, (int)TK_COUNT); k++) h->tune[k] = values[k];
  return DDCSVD_OK;
}

extern "C" int ddcsvd_get_tuning(ddcsvd_handle_t h, int* values, int count) {
  if (!h || !values || count < 0) return DDCSVD_ERR_ARG;
  std::lock_guard<std::mutex> g(h->mu);
  for (int k = 0; k < std::min(count, (int)TK_COUNT); k++) values[k] = h->tune[k];
  return DDCSVD_OK;
}

extern "C" int ddcsvd_autotune_svd(ddcsvd_handle_t h, int m, int n, int mode, int reps) {
  if (!h || m <= 0 || n <= 0 || reps <= 0) return DDCSVD_ERR_ARG;
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  const int k = std::min(m, n);
  const int lda = (int)round_up(m, 4), ldu = lda, ldv = (int)round_up(n, 4);
  float* buf = nullptr;
  const size_t na = (size_t)lda * n, nu = (size_t)ldu * k, nv = (size_t)ldv * k;
  DDC_CUDA_TRY(cudaMalloc((void**)&buf, sizeof(float) * (na + nu + nv + k + 64)));
  float* dA = buf;
  float* dU = dA + na;
  float* dV = dU + nu;
  float* dS = dV + nv;
  fill_uniform_kernel<<<4 * h->num_sms, 256, 0, h->stream>>>(dA, na, 1234567u);
  count_launch();
  std::vector<Candidates> space = {{TK_SPLITK_MAX, {1, 2, 4, 8, 16}}, {TK_TC_BN, {0, 64}},
                                   {TK_PANEL_TAIL, {0, 256, 512, 768}}};
  if (std::max(m, n) >= 2 * std::min(m, n)) space.push_back({TK_TALL_QR, {0, 1}});
  const int rc = coordinate_search(h, space, reps, [&]() {
    return ddcsvd_svd_f32_device(h, m, n, dA, lda, dS, dU, ldu, dV, ldv, mode);
  });
  cudaFree(buf);
  return rc;
}

extern "C" int ddcsvd_autotune_batched(ddcsvd_handle_t h, int batch, const int* m, const int* n, int reps) {
  if (!h || batch <= 0 || !m || !n || reps <= 0) return DDCSVD_ERR_ARG;
  DDC_CUDA_TRY(cudaSetDevice(h->device));
  std::vector<long long> offA(batch), offS(batch), offU(batch), offV(batch);
  long long a = 0, sN = 0, u = 0, v = 0;
  for (int b = 0; b < batch; b++) {
    if (m[b] <= 0 || n[b] <= 0) return DDCSVD_ERR_ARG;
    const long long k = std::min(m[b], n[b]);
    offA[b] = a; a += (long long)m[b] * n[b];
    offS[b] = sN; sN += k;
    offU[b] = u; u += (long long)m[b] * k;
    offV[b] = v; v += (long long)n[b] * k;
  }
  float* buf = nullptr;
  DDC_CUDA_TRY(cudaMalloc((void**)&buf, sizeof(float) * (size_t)(a + sN + u + v + 64)));
  float* dA = buf;
  float* dS = dA + a;
  float* dU = dS + sN;
  float* dV = dU + u;
  fill_uniform_kernel<<<4 * h->num_sms, 256, 0, h->stream>>>(dA, (size_t)a, 7654321u);
  count_launch();
  std::vector<Candidates> space = {
      {TK_BATCH_THREADS, {256, 512}}, {TK_BATCH_SMEM_FULL, {0, 1}}, {TK_DC_TERMS, {4, 8, 16}}};
  const int rc = coordinate_search(h, space, reps, [&]() {
    return ddcsvd_svd_batched_f32_device(h, batch, m, n, dA, offA.data(), dS, offS.data(), dU, offU.data(), dV,
                                         offV.data());
  });
  cudaFree(buf);
  return rc;
}
