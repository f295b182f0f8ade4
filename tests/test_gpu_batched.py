"""Batched uneven SVDs (one launch sequence) against the FP64 oracle / LAPACK."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def uneven_batch(rng, count, mlo=16, mhi=256, wide=False):
    mats = []
    for _ in range(count):
        m = int(rng.integers(mlo, mhi + 1))
        n = int(rng.integers(8, m + 1))
        A = rng.uniform(-1, 1, (m, n)).astype(np.float32)
        if wide and rng.random() < 0.5:
            A = np.ascontiguousarray(A.T)
        mats.append(A)
    return mats


def check_all(orc, mats, outs):
    for A, (s, U, V) in zip(mats, outs):
        s, U, V = (x.double().cpu().numpy() for x in (s, U, V))
        A64 = A.astype(np.float64)
        st = np.linalg.svd(A64, compute_uv=False)
        met = orc.metrics(A64, s, U, V, st)
        assert np.all(np.diff(s) >= 0)
        assert met["sig_abs"] <= TOL and met["resid"] <= TOL, (A.shape, met)
        assert met["orth_u"] <= TOL and met["orth_v"] <= TOL, (A.shape, met)


def test_batched_uneven(lib, cuda, orc):
    rng = np.random.default_rng(3)
    mats = uneven_batch(rng, 96)
    outs = lib.svd_batched_device([cuda.from_numpy(A).cuda() for A in mats])
    check_all(orc, mats, outs)


def test_batched_mixed_orientation(lib, cuda, orc):
    rng = np.random.default_rng(4)
    mats = uneven_batch(rng, 40, mhi=96, wide=True)
    outs = lib.svd_batched_device([cuda.from_numpy(A).cuda() for A in mats])
    check_all(orc, mats, outs)


def test_batched_structured(lib, cuda, orc):
    rng = np.random.default_rng(5)
    mats = [np.eye(20, dtype=np.float32), np.diag(np.repeat([2.0, 1.0], 16)).astype(np.float32),
            (rng.standard_normal((40, 3)) @ rng.standard_normal((3, 30))).astype(np.float32),
            np.ones((1, 1), np.float32), rng.uniform(-1, 1, (2, 1)).astype(np.float32)]
    outs = lib.svd_batched_device([cuda.from_numpy(A).cuda() for A in mats])
    check_all(orc, mats, outs)


def test_batched_many_trees_with_splits(lib, cuda, orc):
    """Enough problems for the tree-per-CTA D&C (>= 64 trees) with some whose
    bidiagonals split inside the problem (identity, diagonal, block-diagonal):
    the layout prepared while stage 1 runs assumes one block per problem and
    must be redone for these."""
    rng = np.random.default_rng(8)
    mats = uneven_batch(rng, 72, mhi=96)
    for k in range(24):
        n = 8 + (k % 5) * 6
        if k % 3 == 0:
            A = np.eye(n)
        elif k % 3 == 1:
            A = np.diag(np.repeat([3.0, 1.0], n // 2))
        else:
            A = np.zeros((n + 4, n))
            A[:n // 2, :n // 2] = rng.standard_normal((n // 2, n // 2))
            A[n // 2:, n // 2:] = rng.standard_normal((n + 4 - n // 2, n - n // 2))
        mats.append(A.astype(np.float32))
    outs = lib.svd_batched_device([cuda.from_numpy(A).cuda() for A in mats])
    check_all(orc, mats, outs)


def test_batched_matches_single(lib, cuda):
    """The batched and single-matrix paths agree (both against the same input)."""
    rng = np.random.default_rng(6)
    mats = uneven_batch(rng, 12, mhi=128)
    outs = lib.svd_batched_device([cuda.from_numpy(A).cuda() for A in mats])
    for A, (s, _, _) in zip(mats, outs):
        s1, _, _ = lib.svd_device(cuda.from_numpy(A).cuda(), mode="plain")
        assert np.max(np.abs(s.cpu().numpy() - s1.cpu().numpy())) <= 1e-5 * float(s1.max())


def test_batched_config_distribution(lib, cuda):
    """2048 problems drawn like the batched configuration (m in [16,256], n in [8,m]);
    size-independent checks computed on the GPU in FP64."""
    torch = cuda
    rng = np.random.default_rng(3)
    mats = uneven_batch(rng, 2048)
    dev = [torch.from_numpy(A).cuda() for A in mats]
    outs = lib.svd_batched_device(dev)
    worst = {"resid": 0.0, "orth_u": 0.0, "orth_v": 0.0}
    for A, (s, U, V) in zip(dev, outs):
        A64, s, U, V = A.double(), s.double(), U.double(), V.double()
        k = s.shape[0]
        r = float(torch.linalg.norm(A64 - (U * s) @ V.T) / torch.linalg.norm(A64))
        ou = float(torch.linalg.norm(U.T @ U - torch.eye(k, device=U.device, dtype=U.dtype)) / k ** 0.5)
        ov = float(torch.linalg.norm(V.T @ V - torch.eye(k, device=V.device, dtype=V.dtype)) / k ** 0.5)
        worst = {"resid": max(worst["resid"], r), "orth_u": max(worst["orth_u"], ou), "orth_v": max(worst["orth_v"], ov)}
    assert max(worst.values()) <= TOL, worst
