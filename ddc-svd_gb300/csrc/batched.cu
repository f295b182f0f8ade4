// batched.cu -- many uneven SVDs per launch sequence.
#include "internal.hpp"

extern "C" int ddcsvd_svd_batched_f32_device(ddcsvd_handle_t h, int batch, const int* m, const int* n,
                                             const float* dA, const long long* offA, float* dSigma,
                                             const long long* offS, float* dU, const long long* offU,
                                             float* dV, const long long* offV) {
  (void)h; (void)batch; (void)m; (void)n; (void)dA; (void)offA; (void)dSigma; (void)offS; (void)dU;
  (void)offU; (void)dV; (void)offV;
  ddcsvd::set_last_error("batched path not built yet");
  return DDCSVD_ERR_UNSUPPORTED;
}
