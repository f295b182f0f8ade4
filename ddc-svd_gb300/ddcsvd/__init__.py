"""ddcsvd -- Python face of libddcsvd.so (GB300 / sm_103a dense SVD).

The functions mirror the reference's C interface (svd_gpu, bidiag_par) with
numpy host arrays, plus device entry points on torch CUDA tensors.  All
numerical work happens in the CUDA library; this module only marshals
pointers.  Matrices are column-major inside the library: a torch tensor A of
shape (m, n) is passed as the column-major buffer of A (its transpose is
made contiguous), and outputs come back as (m, k) / (n, k) views.
Singular values are ascending, as the reference returns them
(Calculations-Parallel.c:56).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import MODES, DdcsvdError, check, load

__all__ = ["svd_gpu", "bidiag_par", "svd", "Handle", "BatchPlan", "svd_device", "bidiag_device",
           "bdsdc_sigma_device", "bdvec_device", "svd_batched_device", "svd_backward_device",
           "launch_count", "DdcsvdError", "MODES"]


def _mode(mode) -> int:
    return MODES[mode] if isinstance(mode, str) else int(mode)


def _addr(a: np.ndarray) -> int:
    return a.ctypes.data


# ---------------------------------------------------------------- host drop-ins
def svd_gpu(A: np.ndarray, mode="auto"):
    """svd_gpu (svd_gpu.c:53) on a float64 host matrix; returns (sigma, U, V).

    Goes through svd_gpu_ex so that failures raise instead of filling NaN."""
    lib = load()
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    k = min(m, n)
    s = np.zeros(k)
    U = np.zeros((m, k), order="F")
    V = np.zeros((n, k), order="F")
    check(lib.svd_gpu_ex(m, n, _addr(A), _addr(s), _addr(U), _addr(V), _mode(mode)), "svd_gpu")
    return s, U, V


def svd_gpu_void(A: np.ndarray):
    """The exact void drop-in svd_gpu(m, n, A, sigma, U, V) (A is clobbered)."""
    lib = load()
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    k = min(m, n)
    s = np.zeros(k)
    U = np.zeros((m, k), order="F")
    V = np.zeros((n, k), order="F")
    lib.svd_gpu(m, n, _addr(A), _addr(s), _addr(U), _addr(V))
    return s, U, V


def bidiag_par(A: np.ndarray):
    """bidiag_par (bidiag_par.c:34) on a float64 host matrix, any shape.

    Returns (A_reflectors, alpha, beta) in the reference's storage: alpha has
    min(m, n) entries, beta min(m, n) - 1 when m >= n and m when m < n (the
    m x (m+1) upper bidiagonal of a wide matrix, bidiag.c:59-60)."""
    lib = load()
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    mn = min(m, n)
    lb = mn - 1 if m >= n else mn
    al = np.zeros(mn)
    be = np.zeros(max(lb, 1))
    lib.bidiag_par(m, n, _addr(A), _addr(al), _addr(be))
    if np.isnan(al).any():
        raise DdcsvdError(2, "bidiag_par")
    return A, al, be[:lb]


def form_u_par(A_mod: np.ndarray):
    """form_u_par (bidiag_par.c:877) on bidiag_par's reflectors: the full m x m left factor."""
    lib = load()
    A = np.asarray(A_mod, dtype=np.float64, order="F")
    m, n = A.shape
    U = np.zeros((m, m), order="F")
    lib.form_u_par(m, n, _addr(A), _addr(U))
    if np.isnan(U.flat[0]):
        raise DdcsvdError(2, "form_u_par")
    return U


def form_v_par(A_mod: np.ndarray):
    """form_v_par (bidiag_par.c:932) on bidiag_par's reflectors: the full n x n right factor."""
    lib = load()
    A = np.asarray(A_mod, dtype=np.float64, order="F")
    m, n = A.shape
    V = np.zeros((n, n), order="F")
    lib.form_v_par(m, n, _addr(A), _addr(V))
    if np.isnan(V.flat[0]):
        raise DdcsvdError(2, "form_v_par")
    return V


def svd(A: np.ndarray, mode="auto"):
    """FP32 host SVD (A not modified); returns (sigma asc, U (m,k), V (n,k)) as float32."""
    lib = load()
    A = np.asarray(A, dtype=np.float32, order="F")
    m, n = A.shape
    k = min(m, n)
    s = np.zeros(k, dtype=np.float32)
    U = np.zeros((m, k), dtype=np.float32, order="F")
    V = np.zeros((n, k), dtype=np.float32, order="F")
    check(lib.ddcsvd_svd_f32(m, n, _addr(A), m, _addr(s), _addr(U), m, _addr(V), n, _mode(mode)),
          "ddcsvd_svd_f32")
    return s, U, V


def launch_count() -> int:
    return int(load().ddcsvd_kernel_launch_count())


# ---------------------------------------------------------------- device API (torch)
class Handle:
    """Owns a library handle bound to the current device and torch's current stream."""

    def __init__(self, device: int | None = None, stream=None):
        import torch
        lib = load()
        if device is None:
            device = torch.cuda.current_device()
        self.device = device
        h = ctypes.c_void_p()
        check(lib.ddcsvd_create(ctypes.addressof(h), device), "ddcsvd_create")
        self._h = h
        s = stream if stream is not None else torch.cuda.current_stream(device)
        check(lib.ddcsvd_set_stream(self._h, ctypes.c_void_p(s.cuda_stream)), "ddcsvd_set_stream")

    @property
    def ptr(self):
        return self._h

    def stage_timing(self, enable: bool = True) -> None:
        check(load().ddcsvd_set_stage_timing(self._h, int(enable)), "set_stage_timing")

    def stage_times(self) -> list[float]:
        buf = (ctypes.c_float * 4)()
        check(load().ddcsvd_get_stage_times(self._h, ctypes.addressof(buf)), "get_stage_times")
        return [float(x) for x in buf]

    def kernel_times(self, nclass: int = 5):
        """(ms, launches) per kernel class of the last SVD (timing must be on)."""
        ms = (ctypes.c_float * nclass)()
        nl = (ctypes.c_int * nclass)()
        check(load().ddcsvd_get_kernel_times(self._h, ctypes.addressof(ms), ctypes.addressof(nl), nclass),
              "get_kernel_times")
        return [float(x) for x in ms], [int(x) for x in nl]

    TUNING_KNOBS = ("splitk_max", "tc_bn", "batch_threads", "batch_smem_full", "dc_terms", "tall_qr",
                    "panel_fused", "panel_tail")

    @property
    def tuning(self) -> dict:
        """Launch knobs of this handle (see ddcsvd_get_tuning)."""
        buf = (ctypes.c_int * len(self.TUNING_KNOBS))()
        check(load().ddcsvd_get_tuning(self._h, ctypes.addressof(buf), len(buf)), "get_tuning")
        return dict(zip(self.TUNING_KNOBS, (int(x) for x in buf)))

    @tuning.setter
    def tuning(self, values: dict) -> None:
        cur = self.tuning
        cur.update(values)
        buf = (ctypes.c_int * len(self.TUNING_KNOBS))(*[cur[k] for k in self.TUNING_KNOBS])
        check(load().ddcsvd_set_tuning(self._h, ctypes.addressof(buf), len(buf)), "set_tuning")

    LIMITS = ("secular_iterations", "wait_us", "workspace_bytes", "barrier_extra_arrivals")

    @property
    def limits(self) -> dict:
        """Limits of this handle (see ddcsvd_get_limits)."""
        buf = (ctypes.c_longlong * len(self.LIMITS))()
        check(load().ddcsvd_get_limits(self._h, ctypes.addressof(buf), len(buf)), "get_limits")
        return dict(zip(self.LIMITS, (int(x) for x in buf)))

    @limits.setter
    def limits(self, values: dict) -> None:
        cur = self.limits
        cur.update(values)
        buf = (ctypes.c_longlong * len(self.LIMITS))(*[cur[k] for k in self.LIMITS])
        check(load().ddcsvd_set_limits(self._h, ctypes.addressof(buf), len(buf)), "set_limits")

    def release_workspace(self) -> None:
        check(load().ddcsvd_release_workspace(self._h), "release_workspace")

    def autotune_svd(self, m: int, n: int, mode="auto", reps: int = 2) -> dict:
        check(load().ddcsvd_autotune_svd(self._h, m, n, _mode(mode), reps), "autotune_svd")
        return self.tuning

    def autotune_batched(self, shapes, reps: int = 2) -> dict:
        ms = np.ascontiguousarray([s[0] for s in shapes], dtype=np.int32)
        ns = np.ascontiguousarray([s[1] for s in shapes], dtype=np.int32)
        check(load().ddcsvd_autotune_batched(self._h, len(ms), _addr(ms), _addr(ns), reps), "autotune_batched")
        return self.tuning

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            load().ddcsvd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_handles: dict = {}


def _handle(h: Handle | None) -> Handle:
    if h is not None:
        return h
    import torch
    dev = torch.cuda.current_device()
    key = (dev, torch.cuda.current_stream(dev).cuda_stream)
    if key not in _default_handles:
        _default_handles[key] = Handle(dev)
    return _default_handles[key]


def colmajor(A):
    """Column-major storage of a (m, n) torch tensor: returns (buffer (n, m) contiguous, ld)."""
    Ac = A.t().contiguous()
    return Ac, A.shape[0]


def svd_device(A, mode="auto", handle: Handle | None = None, out=None):
    """SVD of a float32 CUDA tensor (m, n).  Returns (sigma (k,), U (m, k), V (n, k)).

    `out` = (s, Ut, Vt) with Ut of shape (k, m) and Vt of shape (k, n)
    (the column-major buffers) lets a caller reuse output memory."""
    import torch
    h = _handle(handle)
    m, n = A.shape
    k = min(m, n)
    Ac, lda = colmajor(A)
    if out is None:
        s = torch.empty(k, dtype=torch.float32, device=A.device)
        Ut = torch.empty((k, m), dtype=torch.float32, device=A.device)
        Vt = torch.empty((k, n), dtype=torch.float32, device=A.device)
    else:
        s, Ut, Vt = out
    check(load().ddcsvd_svd_f32_device(h.ptr, m, n, Ac.data_ptr(), lda, s.data_ptr(), Ut.data_ptr(), m,
                                       Vt.data_ptr(), n, _mode(mode)), "ddcsvd_svd_f32_device")
    return s, Ut.t(), Vt.t()


def svd_device_colmajor(h: Handle, m: int, n: int, Ac, s, Ut, Vt, mode="auto"):
    """Lowest-level device call on prepared column-major buffers (no copies)."""
    check(load().ddcsvd_svd_f32_device(h.ptr, m, n, Ac.data_ptr(), m, s.data_ptr(), Ut.data_ptr(), m,
                                       Vt.data_ptr(), n, _mode(mode)), "ddcsvd_svd_f32_device")


def bidiag_device(A, mode="auto", handle: Handle | None = None):
    """Stage 1 on a float32 CUDA tensor (m >= n).  Returns (W_colmajor (n, ldw), d, e, tauq, taup)."""
    import torch
    h = _handle(handle)
    m, n = A.shape
    ldw = (m + 31) // 32 * 32
    W = torch.zeros((n, ldw), dtype=torch.float32, device=A.device)
    W[:, :m] = A.t()
    d = torch.zeros(n, dtype=torch.float32, device=A.device)
    e = torch.zeros(max(n, 1), dtype=torch.float32, device=A.device)
    tq = torch.zeros(n, dtype=torch.float32, device=A.device)
    tp = torch.zeros(max(n, 1), dtype=torch.float32, device=A.device)
    check(load().ddcsvd_bidiag_f32_device(h.ptr, m, n, W.data_ptr(), ldw, d.data_ptr(), e.data_ptr(),
                                          tq.data_ptr(), tp.data_ptr(), _mode(mode)), "bidiag")
    return W, d, e[: max(n - 1, 0)], tq, tp[: max(n - 1, 0)]


def bdsdc_sigma_device(b1, b2, handle: Handle | None = None):
    """Stage 2: ascending sigma of the N x (N+1) bidiagonal (float64 CUDA tensors, b2 length N)."""
    import torch
    h = _handle(handle)
    N = b1.shape[0]
    s = torch.empty(N, dtype=torch.float64, device=b1.device)
    check(load().ddcsvd_bdsdc_sigma_device(h.ptr, N, b1.contiguous().data_ptr(), b2.contiguous().data_ptr(),
                                           s.data_ptr()), "bdsdc_sigma")
    return s


def bdvec_device(a, b, sigma, handle: Handle | None = None):
    """Stages 3-4: (X, Y) right/left vectors of the N x N bidiagonal, as (N, N) with column k = vector k."""
    import torch
    h = _handle(handle)
    N = a.shape[0]
    Xt = torch.empty((N, N), dtype=torch.float32, device=a.device)
    Yt = torch.empty((N, N), dtype=torch.float32, device=a.device)
    bb = torch.zeros(max(N, 1), dtype=torch.float64, device=a.device)
    bb[: N - 1] = b[: N - 1]
    check(load().ddcsvd_bdvec_device(h.ptr, N, a.contiguous().data_ptr(), bb.data_ptr(),
                                     sigma.contiguous().data_ptr(), Xt.data_ptr(), Yt.data_ptr()), "bdvec")
    return Xt.t(), Yt.t()


class BatchPlan:
    """Device buffers and offset tables for repeated batched SVDs of fixed shapes.

    A (flat, column-major per problem) is filled with `load(mats)`; `run()` is
    the bare C-ABI call (what a benchmark times)."""

    def __init__(self, shapes, device="cuda", handle: Handle | None = None):
        import torch
        self.h = _handle(handle)
        self.ms = np.array([s[0] for s in shapes], dtype=np.int32)
        self.ns = np.array([s[1] for s in shapes], dtype=np.int32)
        ks = np.minimum(self.ms, self.ns).astype(np.int64)
        m64, n64 = self.ms.astype(np.int64), self.ns.astype(np.int64)
        def offs(sizes):
            o = np.zeros(len(sizes), dtype=np.int64)
            o[1:] = np.cumsum(sizes)[:-1]
            return o
        self.offA, self.offS = offs(m64 * n64), offs(ks)
        self.offU, self.offV = offs(m64 * ks), offs(n64 * ks)
        self.ks = ks
        self.A = torch.empty(int((m64 * n64).sum()), dtype=torch.float32, device=device)
        self.S = torch.empty(int(ks.sum()), dtype=torch.float32, device=device)
        self.U = torch.empty(int((m64 * ks).sum()), dtype=torch.float32, device=device)
        self.V = torch.empty(int((n64 * ks).sum()), dtype=torch.float32, device=device)

    def load(self, mats):
        import torch
        self.A.copy_(torch.cat([a.t().contiguous().reshape(-1) for a in mats]))

    def run(self):
        check(load().ddcsvd_svd_batched_f32_device(
            self.h.ptr, len(self.ms), _addr(self.ms), _addr(self.ns), self.A.data_ptr(), _addr(self.offA),
            self.S.data_ptr(), _addr(self.offS), self.U.data_ptr(), _addr(self.offU), self.V.data_ptr(),
            _addr(self.offV)), "svd_batched")

    def result(self, b):
        m, n, k = int(self.ms[b]), int(self.ns[b]), int(self.ks[b])
        s = self.S[self.offS[b]: self.offS[b] + k]
        U = self.U[self.offU[b]: self.offU[b] + m * k].view(k, m).t()
        V = self.V[self.offV[b]: self.offV[b] + n * k].view(k, n).t()
        return s, U, V


def svd_batched_device(mats, handle: Handle | None = None):
    """Batched SVD of a list of float32 CUDA tensors of uneven shapes (one launch sequence).

    Returns a list of (sigma, U, V) like svd_device."""
    import torch
    h = _handle(handle)
    B = len(mats)
    ms = np.array([a.shape[0] for a in mats], dtype=np.int32)
    ns = np.array([a.shape[1] for a in mats], dtype=np.int32)
    ks = np.minimum(ms, ns)
    offA = np.zeros(B, dtype=np.int64)
    offS = np.zeros(B, dtype=np.int64)
    offU = np.zeros(B, dtype=np.int64)
    offV = np.zeros(B, dtype=np.int64)
    offA[1:] = np.cumsum(ms.astype(np.int64) * ns)[:-1]
    offS[1:] = np.cumsum(ks.astype(np.int64))[:-1]
    offU[1:] = np.cumsum(ms.astype(np.int64) * ks)[:-1]
    offV[1:] = np.cumsum(ns.astype(np.int64) * ks)[:-1]
    dev = mats[0].device
    A = torch.cat([a.t().contiguous().reshape(-1) for a in mats])
    S = torch.empty(int(ks.sum()), dtype=torch.float32, device=dev)
    U = torch.empty(int((ms.astype(np.int64) * ks).sum()), dtype=torch.float32, device=dev)
    V = torch.empty(int((ns.astype(np.int64) * ks).sum()), dtype=torch.float32, device=dev)
    check(load().ddcsvd_svd_batched_f32_device(h.ptr, B, _addr(ms), _addr(ns), A.data_ptr(), _addr(offA),
                                               S.data_ptr(), _addr(offS), U.data_ptr(), _addr(offU),
                                               V.data_ptr(), _addr(offV)), "svd_batched")
    out = []
    for b in range(B):
        m, n, k = int(ms[b]), int(ns[b]), int(ks[b])
        s = S[offS[b]: offS[b] + k]
        Ub = U[offU[b]: offU[b] + m * k].view(k, m).t()
        Vb = V[offV[b]: offV[b] + n * k].view(k, n).t()
        out.append((s, Ub, Vb))
    return out


def gemm_nt_device(A, B, mode="tf32x6", C=None, alpha=1.0, beta=0.0, handle: Handle | None = None):
    """C = beta*C + alpha * A @ B.T on the library's GEMM back ends (float32 CUDA tensors,
    A (M, K) and B (N, K) row-major).  Returns C as an (M, N) tensor."""
    import torch
    h = _handle(handle)
    M, K = A.shape
    N = B.shape[0]
    Ct = torch.zeros((N, M), dtype=torch.float32, device=A.device) if C is None else C.t().contiguous()
    check(load().ddcsvd_gemm_f32_device(h.ptr, _mode(mode), M, N, K, A.contiguous().data_ptr(), K,
                                        B.contiguous().data_ptr(), K, Ct.data_ptr(), M, alpha, beta), "gemm")
    return Ct.t()


def svd_backward_device(U, S, V, gU, gS, gV, handle: Handle | None = None):
    """Adjoint of the thin SVD for a batch: U (B, m, k), S (B, k), V (B, n, k) -> gA (B, m, n)."""
    import torch
    h = _handle(handle)
    Bt, m, k = U.shape
    n = V.shape[1]
    dt = U.dtype
    fn = load().ddcsvd_svd_backward_f64_device if dt == torch.float64 else load().ddcsvd_svd_backward_f32_device

    def cm(x):  # (B, r, c) -> column-major per matrix
        return None if x is None else x.transpose(1, 2).contiguous()

    Uc, Vc = cm(U), cm(V)
    gUc, gVc = cm(gU), cm(gV)
    Sc = S.contiguous()
    gSc = None if gS is None else gS.contiguous()
    gA = torch.empty((Bt, n, m), dtype=dt, device=U.device)
    ptr = lambda x: 0 if x is None else x.data_ptr()  # noqa: E731
    check(fn(h.ptr, Bt, m, n, ptr(Uc), ptr(Sc), ptr(Vc), ptr(gUc), ptr(gSc), ptr(gVc), gA.data_ptr()),
          "svd_backward")
    return gA.transpose(1, 2)
