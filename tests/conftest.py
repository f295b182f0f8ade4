import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "ddc-svd_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103) and the built library")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build(with_ref=False)
    return oracle


@pytest.fixture(scope="session")
def lib():
    import ddcsvd
    from ddcsvd.build import build
    build()
    return ddcsvd


@pytest.fixture(scope="session")
def cuda(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    torch.cuda.set_device(0)
    return torch


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_names(prefix):
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith(prefix) and f.endswith(".npz"))


def graded(n, seed=1, m=None, cond_exp=6.0):
    """A = Q1 diag(sigma) Q2^T with Haar Q1, Q2 (QR of seeded Gaussians, sign-fixed) and
    sigma_i = 10^(-cond_exp * i / (n-1)); returns (A float64, sigma descending)."""
    m = n if m is None else m
    rng = np.random.default_rng(seed)
    Q1, R1 = np.linalg.qr(rng.standard_normal((m, n)))
    Q1 = Q1 * np.sign(np.diag(R1))
    Q2, R2 = np.linalg.qr(rng.standard_normal((n, n)))
    Q2 = Q2 * np.sign(np.diag(R2))
    s = 10.0 ** (-cond_exp * np.arange(n) / max(n - 1, 1))
    return (Q1 * s) @ Q2.T, s
