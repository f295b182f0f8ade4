"""Bounded failure paths, made to run out on purpose (GPU, through the C ABI).

The reference has no error path: it aborts the process on any failure
(svd_gpu.c:85, cl-helper.h:47-55), caps its secular Newton iteration at 30
but searches its bisection bracket with an unbounded `while (gamma_max < 0)`
(Calculations-Parallel.c:125, 208, 300).  This library bounds every
iteration and every device-side wait and reports a status instead; these
tests make each bound run out through the handle's limits
(ddcsvd_set_limits) and check the status, that the call returns promptly,
and that the handle still gives correct results afterwards.  Nothing here
faults, traps or hangs the GPU: the timeout test makes the first grid
barrier of a cooperative launch wait for one arrival that never comes, with
a 2 ms limit, and the kernel returns on its own.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEFAULTS = {"secular_iterations": 80, "wait_us": 0, "workspace_bytes": 0, "barrier_extra_arrivals": 0}


@pytest.fixture
def handle(lib, cuda):
    h = lib.Handle()
    yield h
    cuda.cuda.synchronize()
    h.close()


def _bidiagonal(N, seed):
    rng = np.random.default_rng(seed)
    b1 = rng.uniform(0.2, 2.0, N)
    b2 = rng.uniform(0.2, 2.0, N)
    b2[-1] = 0.0
    return b1, b2


def _svd_ok(lib, torch, h, A, mode):
    s, U, V = lib.svd_device(torch.from_numpy(A).cuda(), mode=mode, handle=h)
    torch.cuda.synchronize()
    s, U, V = (x.double().cpu().numpy() for x in (s, U, V))
    A64 = A.astype(np.float64)
    st = np.sort(np.linalg.svd(A64, compute_uv=False))
    assert np.max(np.abs(s - st)) <= 1e-5 * st[-1]
    assert np.linalg.norm(A64 - (U * s) @ V.T) <= 1e-5 * np.linalg.norm(A64)


def test_limits_round_trip_and_range_check(lib, handle):
    assert handle.limits == DEFAULTS
    handle.limits = {"secular_iterations": 7, "wait_us": 1234, "workspace_bytes": 1 << 30}
    assert handle.limits == {**DEFAULTS, "secular_iterations": 7, "wait_us": 1234, "workspace_bytes": 1 << 30}
    for bad in ({"secular_iterations": 0}, {"secular_iterations": 81}, {"wait_us": -1},
                {"barrier_extra_arrivals": 5000}):
        with pytest.raises(lib.DdcsvdError) as ei:
            handle.limits = bad
        assert ei.value.status == 1
    assert handle.limits["secular_iterations"] == 7  # a refused set changes nothing
    handle.limits = DEFAULTS
    assert handle.limits == DEFAULTS


def test_secular_iteration_cap_reports_noconv(lib, cuda, orc, handle):
    """One FP64 iteration per root cannot reach FP64 accuracy from the FP32 start."""
    b1, b2 = _bidiagonal(512, 21)
    db1, db2 = cuda.from_numpy(b1).cuda(), cuda.from_numpy(b2).cuda()
    handle.limits = {"secular_iterations": 1}
    with pytest.raises(lib.DdcsvdError) as ei:
        lib.bdsdc_sigma_device(db1, db2, handle=handle)
    assert ei.value.status == 4
    handle.limits = DEFAULTS
    s = lib.bdsdc_sigma_device(db1, db2, handle=handle).cpu().numpy()
    so = orc.dc_sigma(b1, b2)
    assert np.max(np.abs(s - so)) <= 1e-13 * so.max()


def test_secular_iteration_cap_in_full_svd(lib, cuda, handle):
    rng = np.random.default_rng(22)
    A = rng.uniform(-1, 1, (300, 200)).astype(np.float32)
    handle.limits = {"secular_iterations": 1}
    with pytest.raises(lib.DdcsvdError) as ei:
        lib.svd_device(cuda.from_numpy(A).cuda(), mode="blocked", handle=handle)
    assert ei.value.status == 4
    handle.limits = DEFAULTS
    _svd_ok(lib, cuda, handle, A, "blocked")


def test_grid_barrier_timeout_in_dc_kernel(lib, cuda, orc, handle):
    """A grid barrier of the persistent D&C kernel waits for an arrival that
    never comes: every CTA gives up after the 2 ms limit and the call returns
    DDCSVD_ERR_TIMEOUT."""
    b1, b2 = _bidiagonal(512, 23)
    db1, db2 = cuda.from_numpy(b1).cuda(), cuda.from_numpy(b2).cuda()
    lib.bdsdc_sigma_device(db1, db2, handle=handle)  # warm: workspace and module loaded
    cuda.cuda.synchronize()
    handle.limits = {"wait_us": 2000, "barrier_extra_arrivals": 1}
    t0 = time.perf_counter()
    with pytest.raises(lib.DdcsvdError) as ei:
        lib.bdsdc_sigma_device(db1, db2, handle=handle)
    elapsed = time.perf_counter() - t0
    assert ei.value.status == 5
    assert elapsed < 1.0, elapsed
    handle.limits = DEFAULTS
    s = lib.bdsdc_sigma_device(db1, db2, handle=handle).cpu().numpy()
    so = orc.dc_sigma(b1, b2)
    assert np.max(np.abs(s - so)) <= 1e-13 * so.max()


def test_grid_barrier_timeout_in_panel_kernel(lib, cuda, handle):
    """The same in the bidiagonalisation panel kernel (CUDA-core mode, the
    cluster tail off so that every column goes through the panel kernel): the
    call stops at the bidiagonal read-back with DDCSVD_ERR_TIMEOUT."""
    rng = np.random.default_rng(24)
    A = rng.uniform(-1, 1, (640, 640)).astype(np.float32)
    handle.tuning = {"panel_tail": 0}
    _svd_ok(lib, cuda, handle, A, "blocked")
    handle.limits = {"wait_us": 2000, "barrier_extra_arrivals": 1}
    t0 = time.perf_counter()
    with pytest.raises(lib.DdcsvdError) as ei:
        lib.svd_device(cuda.from_numpy(A).cuda(), mode="blocked", handle=handle)
    elapsed = time.perf_counter() - t0
    assert ei.value.status == 5
    assert elapsed < 1.0, elapsed
    handle.limits = DEFAULTS
    _svd_ok(lib, cuda, handle, A, "blocked")


def test_workspace_limit_reports_alloc(lib, cuda, handle):
    """The handle's workspace budget stands in for a failing device allocation."""
    rng = np.random.default_rng(25)
    A = rng.uniform(-1, 1, (512, 256)).astype(np.float32)
    handle.release_workspace()
    handle.limits = {"workspace_bytes": 1 << 16}
    with pytest.raises(lib.DdcsvdError) as ei:
        lib.svd_device(cuda.from_numpy(A).cuda(), mode="blocked", handle=handle)
    assert ei.value.status == 3
    assert "limit" in str(ei.value)
    handle.limits = DEFAULTS
    _svd_ok(lib, cuda, handle, A, "blocked")
