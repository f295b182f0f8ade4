"""ctypes binding of libddcsvd.so (the C ABI in include/ddcsvd.h).

The binding only loads the CUDA library; there is no CPU fallback.  If the
library is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import re

from .build import INCLUDE, LIB_PATH

c_int, c_ll, c_float, c_double, c_void_p = (ctypes.c_int, ctypes.c_longlong, ctypes.c_float,
                                            ctypes.c_double, ctypes.c_void_p)
P = c_void_p  # every pointer crosses the ABI as an untyped address

MODES = {"auto": 0, "plain": 1, "blocked": 2, "tf32x3": 3, "bf16x3": 4, "tf32x6": 5}
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "allocation failed",
          4: "did not converge", 5: "device wait timed out", 6: "no usable device",
          7: "input holds NaN or Inf", 8: "unsupported"}

_SIGS = {
    "svd_gpu": (None, [c_int, c_int, P, P, P, P]),
    "bidiag_par": (None, [c_int, c_int, P, P, P]),
    "form_u_par": (None, [c_int, c_int, P, P]),
    "form_v_par": (None, [c_int, c_int, P, P]),
    "svd_gpu_ex": (c_int, [c_int, c_int, P, P, P, P, c_int]),
    "ddcsvd_svd_f32": (c_int, [c_int, c_int, P, c_int, P, P, c_int, P, c_int, c_int]),
    "ddcsvd_svd_f32_host": (c_int, [P, c_int, c_int, P, c_int, P, P, c_int, P, c_int, c_int]),
    "ddcsvd_create": (c_int, [P, c_int]),
    "ddcsvd_destroy": (c_int, [P]),
    "ddcsvd_set_stream": (c_int, [P, P]),
    "ddcsvd_release_workspace": (c_int, [P]),
    "ddcsvd_svd_f32_device": (c_int, [P, c_int, c_int, P, c_int, P, P, c_int, P, c_int, c_int]),
    "ddcsvd_bidiag_f32_device": (c_int, [P, c_int, c_int, P, c_int, P, P, P, P, c_int]),
    "ddcsvd_bdsdc_sigma_device": (c_int, [P, c_int, P, P, P]),
    "ddcsvd_bdvec_device": (c_int, [P, c_int, P, P, P, P, P]),
    "ddcsvd_split_plan": (c_int, [c_int, P, P, ctypes.c_double, P, P]),
    "ddcsvd_dc_plan": (c_int, [c_int, c_int, P, c_int, P, ctypes.c_longlong, P]),
    "ddcsvd_svd_batched_f32_device": (c_int, [P, c_int, P, P, P, P, P, P, P, P, P, P]),
    "ddcsvd_svd_backward_f64_device": (c_int, [P, c_int, c_int, c_int, P, P, P, P, P, P, P]),
    "ddcsvd_svd_backward_f32_device": (c_int, [P, c_int, c_int, c_int, P, P, P, P, P, P, P]),
    "ddcsvd_svd_backward_f64_noalloc": (c_int, [P, c_int, c_int, c_int, P, P, P, P, P, P, P]),
    "ddcsvd_gemm_f32_device": (c_int, [P, c_int, c_int, c_int, c_int, P, c_int, P, c_int, P, c_int, c_float,
                                       c_float]),
    "ddcsvd_status_string": (ctypes.c_char_p, [c_int]),
    "ddcsvd_last_error": (ctypes.c_char_p, []),
    "ddcsvd_kernel_launch_count": (c_ll, []),
    "ddcsvd_set_stage_timing": (c_int, [P, c_int]),
    "ddcsvd_get_tuning": (c_int, [P, P, c_int]),
    "ddcsvd_set_limits": (c_int, [P, P, c_int]),
    "ddcsvd_get_limits": (c_int, [P, P, c_int]),
    "ddcsvd_set_tuning": (c_int, [P, P, c_int]),
    "ddcsvd_autotune_svd": (c_int, [P, c_int, c_int, c_int, c_int]),
    "ddcsvd_autotune_batched": (c_int, [P, c_int, P, P, c_int]),
    "ddcsvd_get_stage_times": (c_int, [P, P]),
    "ddcsvd_get_kernel_times": (c_int, [P, P, P, c_int]),
}

_lib = None


class DdcsvdError(RuntimeError):
    def __init__(self, status: int, where: str = ""):
        detail = ""
        if _lib is not None:
            detail = (_lib.ddcsvd_last_error() or b"").decode(errors="replace")
        super().__init__(f"{where}: {STATUS.get(status, status)} ({detail})")
        self.status = status


def header_symbols() -> list[str]:
    """Function names declared in include/ddcsvd.h."""
    text = open(os.path.join(INCLUDE, "ddcsvd.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text)) - {"defined"})


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"libddcsvd.so not built ({path}); run __graft_entry__.build()")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status: int, where: str) -> None:
    if status != 0:
        raise DdcsvdError(status, where)
