"""Generates tests/golden/*.npz from the reference's own host C code.

Run on a machine that has the reference sources (the build reads them in
place through oracle/Makefile's `ref` target; DDCSVD_REF_SRC names their
directory):

    python tests/golden/make_golden.py

Each fixture stores the input matrix and the reference's outputs on it:
  * bidiag_*.npz : A, alpha, beta, A_refl (bidiag_seq, bidiag.c:33-186)
  * svd_*.npz    : A, sigma (ascending), U, V, alpha, beta, X, Y from the
                   svd_gpu stage order (svd_gpu.c:99-121) with bidiag_seq,
                   plus sigma_lapack (numpy FP64 LAPACK) for context.
Inputs are seeded numpy draws, except `svd_twsvd_*`, which reproduces
test-whole-svd.c's own input: glibc rand() with its default seed 1,
A[i] = 1 + 3 * rand() / (RAND_MAX + 1.0) in column-major order
(test-whole-svd.c:18-23, 69-71), and `svd_cfg_512x256`, the plain
single-matrix configuration exactly: default_rng(0).uniform(-1, 1,
(512, 256)) rounded to FP32 (the reference runs on those FP32 values in
FP64).  Its V is the reference's and wrong (multV's leading dimension for
m != n); tests compare sigma and U only.

    python tests/golden/make_golden.py --only svd_cfg_512x256   # one fixture
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def glibc_rand_matrix(m: int, n: int) -> np.ndarray:
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    RAND_MAX = 2147483647
    vals = np.array([libc.rand() for _ in range(m * n)], dtype=np.float64)
    a = 1.0 + 3.0 * vals / (RAND_MAX + 1.0)
    return a.reshape((n, m)).T.copy(order="F")


REF_SRC = os.environ.get("DDCSVD_REF_SRC", "/root/reference")


def main(only: list[str] | None = None) -> None:
    O.build(with_ref=True, ref_src=REF_SRC)
    out = {}
    rng = np.random.default_rng(20121220)
    # bidiagonalisation goldens, including the m < n edge path (bidiag.c:133-160)
    for (m, n) in [(8, 8), (17, 17), (33, 20), (64, 64), (100, 37), (20, 33), (128, 128), (5, 2), (2, 5), (1, 1), (3, 1)]:
        A = rng.uniform(1.0, 2.0, (m, n))  # bidiag_dr.c:92-93 draws U[1,2)
        Ar, al, be = O.ref_bidiag(A)
        out[f"bidiag_{m}x{n}"] = dict(A=A, alpha=al, beta=be, A_refl=Ar)
    # full-pipeline goldens (square: the reference's V is wrong for m != n)
    cases = [("u14", 8, 8), ("u14", 32, 32), ("u14", 64, 64), ("um11", 96, 96),
             ("u14", 128, 128), ("um11", 256, 256), ("um11", 64, 32)]
    for kind, m, n in cases:
        if kind == "u14":
            A = rng.uniform(1.0, 4.0, (m, n))
        else:
            A = rng.uniform(-1.0, 1.0, (m, n))
        r = O.ref_svd(A)
        out[f"svd_{kind}_{m}x{n}"] = dict(
            A=A, sigma=r["sigma"], U=r["U"].astype(np.float32), V=r["V"].astype(np.float32),
            alpha=r["alpha"], beta=r["beta"], X=r["X"].astype(np.float32),
            Y=r["Y"].astype(np.float32), sigma_lapack=np.linalg.svd(A, compute_uv=False)[::-1].copy())
    A = glibc_rand_matrix(48, 48)
    r = O.ref_svd(A)
    out["svd_twsvd_48x48"] = dict(A=A, sigma=r["sigma"], U=r["U"].astype(np.float32),
                                  V=r["V"].astype(np.float32), alpha=r["alpha"], beta=r["beta"],
                                  X=r["X"].astype(np.float32), Y=r["Y"].astype(np.float32),
                                  sigma_lapack=np.linalg.svd(A, compute_uv=False)[::-1].copy())
    # the plain single-matrix configuration: 512 x 256, U[-1, 1] from default_rng(0), FP32 entries
    A = np.random.default_rng(0).uniform(-1.0, 1.0, (512, 256)).astype(np.float32).astype(np.float64)
    r = O.ref_svd(A)
    out["svd_cfg_512x256"] = dict(A=A, sigma=r["sigma"], U=r["U"].astype(np.float32), V=r["V"].astype(np.float32),
                                  alpha=r["alpha"], beta=r["beta"],
                                  sigma_lapack=np.linalg.svd(A, compute_uv=False)[::-1].copy())
    written = 0
    for name, d in out.items():
        if only and name not in only:
            continue
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        written += 1
    print(f"wrote {written} fixtures to {HERE}")


if __name__ == "__main__":
    main(sys.argv[sys.argv.index("--only") + 1:] if "--only" in sys.argv else None)
