"""CPU tests of the C ABI boundary: the library builds for sm_103a, loads, exports
every function include/ddcsvd.h declares, and fails loudly without a GPU."""
import ctypes

import pytest


def test_library_exports_every_header_symbol(lib):
    from ddcsvd import _lib
    L = lib.load()
    syms = _lib.header_symbols()
    assert "svd_gpu" in syms and "bidiag_par" in syms
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_binding_covers_header(lib):
    from ddcsvd import _lib
    assert set(_lib.header_symbols()) <= set(_lib._SIGS), set(_lib.header_symbols()) - set(_lib._SIGS)


def test_status_strings(lib):
    L = lib.load()
    assert L.ddcsvd_status_string(0) == b"ok"
    assert L.ddcsvd_status_string(7) == b"input holds NaN or Inf"
    assert L.ddcsvd_status_string(99) == b"unknown status"


def test_argument_validation_needs_no_gpu(lib):
    L = lib.load()
    assert L.ddcsvd_svd_f32(0, 4, None, 4, None, None, 4, None, 4, 0) == 1
    assert L.ddcsvd_svd_f32_device(None, 4, 4, None, 4, None, None, 4, None, 4, 0) == 1
    assert L.ddcsvd_create(None, 0) == 1


def test_no_device_is_reported_not_faked(lib):
    import numpy as np
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(lib.DdcsvdError) as ei:
        lib.svd(np.eye(4, dtype=np.float32))
    assert ei.value.status in (2, 6)


def test_cubin_targets_sm103a(lib):
    import subprocess
    from ddcsvd.build import LIB_PATH
    out = subprocess.run(["cuobjdump", "--list-elf", LIB_PATH], capture_output=True, text=True).stdout
    assert "sm_103a" in out
