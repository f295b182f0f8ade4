"""CPU checkers for the ddc-svd GPU library -- TEST INFRASTRUCTURE ONLY.

Loads two shared libraries built by ``oracle/Makefile``:

* ``_build/libddcsvd_oracle.so`` -- our FP64 restatement of the reference
  pipeline (``ddcsvd_oracle.c``; each function cites the reference file:line
  it follows);
* ``_ref/libddcsvd_ref.so`` -- the reference's own host C code compiled from
  its sources (only where the reference sources were available at build
  time).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module.  The product library never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libddcsvd_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libddcsvd_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)


def build(with_ref: bool | None = None, ref_src: str | None = None) -> None:
    """Compile the oracle (always) and the reference build from the reference's
    sources in `ref_src` (else the DDCSVD_REF_SRC environment variable): when
    with_ref is True, or None and that directory exists."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    src = ref_src or os.environ.get("DDCSVD_REF_SRC", "")
    if with_ref is None:
        with_ref = bool(src) and os.path.isdir(src)
    if with_ref:
        if not (src and os.path.isdir(src)):
            raise RuntimeError("the reference build needs its sources: pass ref_src or set DDCSVD_REF_SRC")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={src}"], check=True)


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["F_CONTIGUOUS"] or a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_ref=False)
        _lib = ctypes.CDLL(ORACLE_SO)
        i, p = ctypes.c_int, _dp
        _lib.orc_bidiag.argtypes = [i, i, p, i, p, p]
        _lib.orc_dc_sigma.argtypes = [i, p, p, p]
        _lib.orc_twisted.argtypes = [i, p, p, p, p]
        _lib.orc_left.argtypes = [i, p, p, p, p, p]
        _lib.orc_svd.argtypes = [i, i, p, i, p, p, i, p, i, p, p, p, p]
        _lib.orc_bdsvd.argtypes = [i, p, p, ctypes.c_double, p, p]
        _lib.orc_bidiag_steps.argtypes = [i, i, p, i, p, p, i]
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_SO)
        i, p = ctypes.c_int, _dp
        _ref.ref_svd.argtypes = [i, i, p, p, p, p, p, p, p, p, p]
        _ref.ref_bidiag.argtypes = [i, i, p, p, p]
    return _ref


# ---------------------------------------------------------------- oracle
def bidiag(A: np.ndarray):
    """Reference-convention bidiagonalisation (bidiag.c:33). Returns (A_refl, alpha, beta)."""
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    mn = min(m, n)
    alpha = np.zeros(mn)
    beta = np.zeros(mn)
    rc = lib().orc_bidiag(m, n, _ptr(A), m, _ptr(alpha), _ptr(beta))
    assert rc == 0
    lb = mn - 1 if m >= n else mn
    return A, alpha, beta[:lb]


def bidiag_steps(A: np.ndarray, steps: int) -> None:
    """Runs the first `steps` Householder steps of the reference bidiagonalisation
    in place on A (float64, Fortran order) -- a bounded timing sample."""
    assert A.dtype == np.float64 and A.flags["F_CONTIGUOUS"]
    m, n = A.shape
    al = np.zeros(min(m, n))
    be = np.zeros(min(m, n))
    assert lib().orc_bidiag_steps(m, n, _ptr(A), m, _ptr(al), _ptr(be), int(steps)) == 0


def dc_sigma(b1: np.ndarray, b2: np.ndarray) -> np.ndarray:
    """Ascending singular values of the N x (N+1) bidiagonal (b2[N-1] = 0 for N x N)."""
    b1 = np.ascontiguousarray(b1, dtype=np.float64)
    N = b1.shape[0]
    bb = np.zeros(N)
    bb[: len(b2)] = b2
    s = np.zeros(N)
    assert lib().orc_dc_sigma(N, _ptr(b1), _ptr(bb), _ptr(s)) == 0
    return s


def twisted(a: np.ndarray, b: np.ndarray, sigma: np.ndarray) -> np.ndarray:
    """Right vectors of the N x N bidiagonal; returns X with X[:, k] = x_k."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    N = a.shape[0]
    bb = np.zeros(max(N, 1))
    bb[: N - 1] = b[: N - 1]
    s = np.ascontiguousarray(sigma, dtype=np.float64)
    X = np.zeros((N, N))  # row k = vector k (C order)
    assert lib().orc_twisted(N, _ptr(a), _ptr(bb), _ptr(s), _ptr(X)) == 0
    return X.T.copy()


def bdsvd(a: np.ndarray, b: np.ndarray, eps: float = float(np.finfo(np.float64).eps)):
    """Singular values (ascending) and right vectors of the N x N bidiagonal with
    splitting at negligible b (tolerance 4 eps max|B|).  Returns (sigma, X, b_split)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    N = a.shape[0]
    bb = np.zeros(max(N, 1))
    bb[: N - 1] = b[: N - 1]
    s = np.zeros(N)
    X = np.zeros((N, N))
    assert lib().orc_bdsvd(N, _ptr(a), _ptr(bb), eps, _ptr(s), _ptr(X)) == 0
    return s, X.T.copy(), bb[: N - 1]


def svd(A: np.ndarray, stages: bool = False):
    """Full FP64 pipeline. Returns (sigma ascending, U m x mn, V n x mn[, stages dict])."""
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    mn = min(m, n)
    s = np.zeros(mn)
    U = np.zeros((m, mn), order="F")
    V = np.zeros((n, mn), order="F")
    al = np.zeros(mn)
    be = np.zeros(mn)
    X = np.zeros((mn, mn))
    Y = np.zeros((mn, mn))
    rc = lib().orc_svd(m, n, _ptr(A), m, _ptr(s), _ptr(U), m, _ptr(V), n,
                       _ptr(al), _ptr(be), _ptr(X), _ptr(Y))
    assert rc == 0
    if stages:
        return s, U, V, {"alpha": al, "beta": be[: mn - 1], "X": X.T.copy(), "Y": Y.T.copy()}
    return s, U, V


# ---------------------------------------------------------------- reference
def ref_svd(A: np.ndarray):
    """The reference's own host pipeline (bidiag_seq + host stages).

    Returns dict with sigma (ascending), U, V, alpha, beta, X, Y (columns are
    vectors), t_stage (seconds per stage).  V is wrong for m != n (a defect
    of the reference's multV, bidiag_par.c:1034-1036)."""
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    mn = min(m, n)
    lb = mn - 1 if m >= n else mn
    s = np.zeros(mn)
    U = np.zeros((m, mn), order="F")
    V = np.zeros((n, mn), order="F")
    al = np.zeros(mn)
    be = np.zeros(max(lb, 1))
    X = np.zeros((mn, lb + 1))
    Y = np.zeros((mn, mn))
    t = np.zeros(5)
    rc = ref().ref_svd(m, n, _ptr(A), _ptr(s), _ptr(U), _ptr(V), _ptr(al), _ptr(be),
                       _ptr(X), _ptr(Y), _ptr(t))
    assert rc == 0
    return {"sigma": s, "U": U, "V": V, "alpha": al, "beta": be[:lb], "X": X.T.copy(),
            "Y": Y.T.copy(), "t_stage": t, "A_refl": A}


def ref_bidiag(A: np.ndarray):
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = A.shape
    mn = min(m, n)
    lb = mn - 1 if m >= n else mn
    al = np.zeros(mn)
    be = np.zeros(max(lb, 1))
    assert ref().ref_bidiag(m, n, _ptr(A), _ptr(al), _ptr(be)) == 0
    return A, al, be[:lb]


# ---------------------------------------------------------------- metrics
def metrics(A: np.ndarray, sigma: np.ndarray, U: np.ndarray, V: np.ndarray,
            sigma_true: np.ndarray | None = None) -> dict:
    """Accuracy figures reported for every result (FP64 arithmetic).

    resid   = ||A - U diag(s) V^T||_F / ||A||_F
    orth_u  = ||U^T U - I||_F / sqrt(k)   (RMS column-pair error; k = #vectors)
    orth_v  = ||V^T V - I||_F / sqrt(k)
    sig_rel = max_i |s_i - s_i*| / s_i*   (when the true values are given)
    sig_abs = max_i |s_i - s_i*| / s_max*
    """
    A = np.asarray(A, dtype=np.float64)
    s = np.asarray(sigma, dtype=np.float64)
    U = np.asarray(U, dtype=np.float64)
    V = np.asarray(V, dtype=np.float64)
    k = s.shape[0]
    R = A - (U * s) @ V.T
    out = {
        "resid": float(np.linalg.norm(R) / max(np.linalg.norm(A), 1e-300)),
        "orth_u": float(np.linalg.norm(U.T @ U - np.eye(k)) / np.sqrt(max(k, 1))),
        "orth_v": float(np.linalg.norm(V.T @ V - np.eye(k)) / np.sqrt(max(k, 1))),
    }
    if sigma_true is not None:
        st = np.sort(np.asarray(sigma_true, dtype=np.float64))
        ss = np.sort(s)
        out["sig_rel"] = float(np.max(np.abs(ss - st) / np.maximum(st, 1e-300)))
        out["sig_abs"] = float(np.max(np.abs(ss - st)) / max(st[-1], 1e-300))
    return out
