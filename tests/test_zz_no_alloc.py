"""The allocation-free FP64 SVD adjoint, ddcsvd_svd_backward_f64_noalloc.

Callers that may not allocate device memory when they need the adjoint (code
inside another framework's memory pool or a fixed memory budget, or a loop
that must stay away from the driver's allocator) use this entry point: it
takes no handle and keeps its intermediates in a fixed 16 MiB array inside
the library.  These tests call it through the C ABI and compare it with the
handle-based entry point, ddcsvd_svd_backward_f64_device, on two calls in a
row (the second call finds the first call's data still in the shared array),
check the size limit at exactly its documented value (accepted) and one
problem beyond it (refused), and run a batch larger than one launch grid
holds (more than 65535 problems).  The entry point only enqueues its work on
the given stream; torch's own kernels on that stream run after it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(torch, seed, B, m, n):
    g = torch.Generator(device="cuda").manual_seed(seed)
    U = torch.linalg.qr(torch.randn((B, m, n), dtype=torch.float64, device="cuda", generator=g))[0]
    V = torch.linalg.qr(torch.randn((B, n, n), dtype=torch.float64, device="cuda", generator=g))[0]
    S = (1.0 + torch.arange(n, dtype=torch.float64, device="cuda") / 64.0).repeat(B, 1)
    gU = torch.randn((B, m, n), dtype=torch.float64, device="cuda", generator=g)
    gS = torch.randn((B, n), dtype=torch.float64, device="cuda", generator=g)
    gV = torch.randn((B, n, n), dtype=torch.float64, device="cuda", generator=g)
    return U, S, V, gU, gS, gV


def _noalloc(lib, torch, U, S, V, gU, gS, gV):
    """Calls the C entry point directly with column-major per-problem buffers."""
    B, m, n = U.shape
    cm = lambda x: x.transpose(1, 2).contiguous()  # noqa: E731
    Uc, Vc, gUc, gVc = cm(U), cm(V), cm(gU), cm(gV)
    Sc, gSc = S.contiguous(), gS.contiguous()
    gA = torch.full((B, n, m), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.load().ddcsvd_svd_backward_f64_noalloc(
        ctypes.c_void_p(stream), B, m, n, Uc.data_ptr(), Sc.data_ptr(), Vc.data_ptr(), gUc.data_ptr(),
        gSc.data_ptr(), gVc.data_ptr(), gA.data_ptr())
    return rc, gA.transpose(1, 2)


def test_noalloc_adjoint_matches_handle_entry_point(lib, cuda):
    torch = cuda
    # two calls in a row with different shapes and data
    for seed, (B, m, n) in ((11, (6, 128, 64)), (12, (3, 96, 40))):
        U, S, V, gU, gS, gV = _problem(torch, seed, B, m, n)
        ref = lib.svd_backward_device(U, S, V, gU, gS, gV)
        rc, got = _noalloc(lib, torch, U, S, V, gU, gS, gV)
        assert rc == 0, lib.load().ddcsvd_last_error()
        err = float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref))
        assert err <= 1e-12, err


def test_noalloc_adjoint_without_vector_gradients(lib, cuda):
    torch = cuda
    U, S, V, gU, gS, gV = _problem(torch, 13, 4, 64, 32)
    B, m, n = U.shape
    cm = lambda x: x.transpose(1, 2).contiguous()  # noqa: E731
    gA = torch.empty((B, n, m), dtype=torch.float64, device="cuda")
    rc = lib.load().ddcsvd_svd_backward_f64_noalloc(
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), B, m, n, cm(U).data_ptr(), S.data_ptr(),
        cm(V).data_ptr(), None, gS.contiguous().data_ptr(), None, gA.data_ptr())
    assert rc == 0
    ref = torch.einsum("bij,bj,bkj->bik", U, gS, V)  # d(w^T s)/dA = U diag(w) V^T
    assert float(torch.linalg.norm(gA.transpose(1, 2) - ref) / torch.linalg.norm(ref)) <= 1e-12


def test_noalloc_adjoint_refuses_more_than_its_scratch(lib, cuda):
    torch = cuda
    B, m, n = 64, 256, 128  # 64 * (3*128^2 + 256*128) * 8 bytes > 16 MiB
    U, S, V, gU, gS, gV = _problem(torch, 14, 2, m, n)
    U, V, gU, gV = (x.repeat(B // 2, 1, 1) for x in (U, V, gU, gV))
    S, gS = S.repeat(B // 2, 1), gS.repeat(B // 2, 1)
    rc, _ = _noalloc(lib, torch, U, S, V, gU, gS, gV)
    assert rc == 1
    assert b"limit" in lib.load().ddcsvd_last_error()


def _limit_bytes(B, m, n):
    r = lambda x: (x + 255) // 256 * 256  # noqa: E731
    return 3 * r(8 * B * n * n) + r(8 * B * m * n)


def test_noalloc_adjoint_limit_is_exact(lib, cuda):
    """m = n = 64: each problem takes 128 KiB, so 128 problems fill the 16 MiB exactly."""
    torch = cuda
    m = n = 64
    assert _limit_bytes(128, m, n) == 16 << 20 and _limit_bytes(129, m, n) > 16 << 20
    U, S, V, gU, gS, gV = _problem(torch, 15, 129, m, n)
    rc, got = _noalloc(lib, torch, U[:128], S[:128], V[:128], gU[:128], gS[:128], gV[:128])
    assert rc == 0, lib.load().ddcsvd_last_error()
    ref = lib.svd_backward_device(U[:128], S[:128], V[:128], gU[:128], gS[:128], gV[:128])
    assert float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref)) <= 1e-12
    rc, _ = _noalloc(lib, torch, U, S, V, gU, gS, gV)
    assert rc == 1


def test_noalloc_adjoint_batch_beyond_one_launch_grid(lib, cuda):
    torch = cuda
    B, m, n = 70000, 3, 2
    U, S, V, gU, gS, gV = _problem(torch, 16, B, m, n)
    rc, got = _noalloc(lib, torch, U, S, V, gU, gS, gV)
    assert rc == 0, lib.load().ddcsvd_last_error()
    ref = lib.svd_backward_device(U, S, V, gU, gS, gV)
    assert float(torch.linalg.norm(got - ref) / torch.linalg.norm(ref)) <= 1e-12
    # the last chunk (problems 65535..69999) against a direct evaluation
    k = slice(65535, B)
    Ui, Si, Vi, gUi, gSi, gVi = U[k], S[k], V[k], gU[k], gS[k], gV[k]
    F = Si[:, None, :] ** 2 - Si[:, :, None] ** 2
    F = torch.where(F == 0, torch.full_like(F, float("inf")), F).reciprocal()
    J = Ui.transpose(1, 2) @ gUi
    K = Vi.transpose(1, 2) @ gVi
    Mi = torch.diag_embed(gSi) + (F * (J - J.transpose(1, 2))) * Si[:, None, :] + \
        Si[:, :, None] * (F * (K - K.transpose(1, 2)))
    proj = gUi - Ui @ (Ui.transpose(1, 2) @ gUi)
    direct = Ui @ Mi @ Vi.transpose(1, 2) + (proj / Si[:, None, :]) @ Vi.transpose(1, 2)
    assert float(torch.linalg.norm(got[k] - direct) / torch.linalg.norm(direct)) <= 1e-12
