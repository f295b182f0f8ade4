"""CPU tests of the FP64 oracle: pinned against the reference's own outputs
(tests/golden, produced by oracle/_ref from the reference sources) and LAPACK."""
import numpy as np
import pytest

from conftest import golden, golden_names


@pytest.mark.parametrize("name", golden_names("bidiag_"))
def test_bidiag_matches_reference(orc, name):
    g = golden(name)
    A_r, al, be = orc.bidiag(g["A"])
    scale = np.abs(g["A"]).max()
    assert np.allclose(al, g["alpha"], rtol=0, atol=1e-12 * scale)
    assert np.allclose(be, g["beta"], rtol=0, atol=1e-12 * scale)
    ok = np.isfinite(g["A_refl"])
    assert np.allclose(A_r[ok], g["A_refl"][ok], rtol=0, atol=1e-10)


@pytest.mark.parametrize("name", [g for g in golden_names("bidiag_") if golden(g)["A"].shape[0] < golden(g)["A"].shape[1]])
def test_wide_bidiag_is_tall_bidiag_of_padded_transpose(orc, name):
    """The identity the GPU bidiag_par uses for m < n: the reference's wide
    reduction (bidiag.c:130-155) is the tall reduction of C = [0 | A^T]
    (n x (m+1)) step for step -- alpha_i = e_C[i], beta_i = d_C[i+1],
    A_refl[i, j] = C_refl[j, i+1] -- checked on the reference's own outputs."""
    g = golden(name)
    A = g["A"]
    m, n = A.shape
    C = np.zeros((n, m + 1))
    C[:, 1:] = A.T
    C_r, d, e = orc.bidiag(C)
    scale = np.abs(A).max()
    assert np.allclose(e[:m], g["alpha"], rtol=0, atol=1e-12 * scale)
    assert np.allclose(d[1:m + 1], g["beta"], rtol=0, atol=1e-12 * scale)
    assert np.allclose(C_r[:, 1:].T, g["A_refl"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("name", golden_names("svd_"))
def test_sigma_matches_reference_within_its_accuracy(orc, name):
    g = golden(name)
    s, U, V = orc.svd(g["A"])
    smax = g["sigma_lapack"].max()
    # oracle: FP64 accurate
    assert np.max(np.abs(s - g["sigma_lapack"])) <= 1e-12 * smax
    # reference (D&C stops at |g| <= 1e-5, Calculations-Parallel.c:163): agrees to its own accuracy
    ref = g["sigma"]
    if np.all(np.isfinite(ref)):
        assert np.max(np.abs(s - ref)) <= 1e-4 * smax


@pytest.mark.parametrize("name", golden_names("svd_"))
def test_vectors_match_reference_up_to_sign(orc, name):
    g = golden(name)
    s, U, V = orc.svd(g["A"])
    m, n = g["A"].shape
    Ur = g["U"].astype(np.float64)
    # columns whose singular value is well separated (relative gap > 1e-2) and finite in the reference
    gaps = np.diff(s)
    gap = np.minimum(np.r_[np.inf, gaps], np.r_[gaps, np.inf]) / s.max()
    cols = [k for k in range(len(s)) if gap[k] > 1e-2 and np.all(np.isfinite(Ur[:, k]))]
    assert cols
    for k in cols:
        assert abs(abs(U[:, k] @ Ur[:, k]) / np.linalg.norm(Ur[:, k]) - 1.0) < 1e-3
        if m == n:  # reference V is wrong for m != n (multV leading dimension)
            Vr = g["V"][:, k].astype(np.float64)
            assert abs(abs(V[:, k] @ Vr) / np.linalg.norm(Vr) - 1.0) < 1e-3


@pytest.mark.parametrize("m,n", [(1, 1), (2, 2), (3, 3), (2, 1), (5, 3), (3, 5), (17, 17), (40, 13), (13, 40),
                                 (100, 100), (257, 129)])
def test_oracle_vs_lapack(orc, m, n):
    rng = np.random.default_rng(m * 1000 + n)
    A = rng.uniform(-1, 1, (m, n))
    s, U, V = orc.svd(A)
    st = np.linalg.svd(A, compute_uv=False)
    met = orc.metrics(A, s, U, V, st)
    assert met["resid"] < 1e-13 and met["orth_u"] < 1e-13 and met["orth_v"] < 1e-13, met
    assert met["sig_abs"] < 1e-13, met
    assert np.all(np.diff(s) >= 0)  # ascending, as the reference returns them


@pytest.mark.parametrize("kind", ["identity", "zero", "diag_repeated", "rank_deficient", "graded", "tiny_block"])
def test_oracle_structured(orc, kind):
    from conftest import graded
    n = 48
    rng = np.random.default_rng(7)
    if kind == "identity":
        A = np.eye(n)
    elif kind == "zero":
        A = np.zeros((n, n))
    elif kind == "diag_repeated":
        A = np.diag(np.repeat([3.0, 2.0, 1.0], n // 3))
    elif kind == "rank_deficient":
        A = rng.standard_normal((n, 5)) @ rng.standard_normal((5, n))
    elif kind == "graded":
        A, _ = graded(n)
    else:
        A = np.zeros((n, n))
        A[:8, :8] = rng.standard_normal((8, 8))
        A[8:, 8:] = 1e-9 * rng.standard_normal((n - 8, n - 8))
    s, U, V = orc.svd(A)
    st = np.linalg.svd(A, compute_uv=False)
    assert np.max(np.abs(np.sort(s) - np.sort(st))) <= 1e-12 * max(st.max(), 1.0)
    if kind in ("zero", "rank_deficient"):
        return  # vectors of a repeated zero singular value are not unique
    met = orc.metrics(A, s, U, V, st)
    assert met["resid"] < 1e-12 and met["orth_v"] < 1e-12, met


def test_dc_sigma_rectangular_bidiagonal(orc):
    """N x (N+1) bidiagonal (b2[N-1] != 0), the shape the reference's D&C recursion works on."""
    rng = np.random.default_rng(3)
    for N in (1, 2, 3, 7, 64, 301):
        b1 = rng.uniform(0.5, 2, N)
        b2 = rng.uniform(0.5, 2, N)
        B = np.zeros((N, N + 1))
        B[np.arange(N), np.arange(N)] = b1
        B[np.arange(N), np.arange(N) + 1] = b2
        s = orc.dc_sigma(b1, b2)
        st = np.sort(np.linalg.svd(B, compute_uv=False))
        assert np.max(np.abs(s - st)) <= 1e-13 * st.max()


def test_reference_build_agrees_when_available(orc):
    """Live check against oracle/_ref (only where the reference sources were built)."""
    if not orc.ref_available():
        pytest.skip("reference build not present")
    rng = np.random.default_rng(11)
    A = rng.uniform(-1, 1, (96, 96))
    r = orc.ref_svd(A)
    Ar, al, be = orc.bidiag(A)
    assert np.allclose(al, r["alpha"], atol=1e-12) and np.allclose(be, r["beta"], atol=1e-12)
    s, _, _ = orc.svd(A)
    assert np.max(np.abs(s - r["sigma"])) <= 1e-4 * s.max()
