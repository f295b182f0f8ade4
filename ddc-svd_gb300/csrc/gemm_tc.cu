// gemm_tc.cu -- tcgen05 tensor-core GEMM back ends (split TF32 / split BF16).
#include "internal.hpp"

namespace ddcsvd {

bool tc_available(ddcsvd_context* ctx) {
  (void)ctx;
  return false;
}

size_t gemm_tc_scratch_bytes(GemmKind kind, int M, int N, int K) {
  (void)kind;
  return (size_t)2 * ((size_t)M * K + (size_t)K * N) * sizeof(float) + 4096;
}

int gemm_tc(ddcsvd_context* ctx, GemmKind kind, int M, int N, int K1, Mat A1, Mat B1, int K2, Mat A2,
            Mat B2, float alpha, float beta, float* C, int ldc, Arena* scratch) {
  (void)ctx; (void)kind; (void)M; (void)N; (void)K1; (void)A1; (void)B1; (void)K2; (void)A2; (void)B2;
  (void)alpha; (void)beta; (void)C; (void)ldc; (void)scratch;
  set_last_error("tensor-core GEMM not built");
  return DDCSVD_ERR_UNSUPPORTED;
}

}  // namespace ddcsvd
