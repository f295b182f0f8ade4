// adjoint.cu -- reverse-mode derivative of the thin SVD.
#include "internal.hpp"

extern "C" int ddcsvd_svd_backward_f64_device(ddcsvd_handle_t, int, int, int, const double*, const double*,
                                              const double*, const double*, const double*, const double*,
                                              double*) {
  ddcsvd::set_last_error("adjoint not built yet");
  return DDCSVD_ERR_UNSUPPORTED;
}
extern "C" int ddcsvd_svd_backward_f32_device(ddcsvd_handle_t, int, int, int, const float*, const float*,
                                              const float*, const float*, const float*, const float*,
                                              float*) {
  ddcsvd::set_last_error("adjoint not built yet");
  return DDCSVD_ERR_UNSUPPORTED;
}
