"""GPU parity tests: the CUDA library (through its C ABI) against the FP64
oracle, LAPACK, and the reference's own outputs (tests/golden).

Tolerances (FP32 pipeline, FP64 singular-value and bidiagonal-vector stages):
  sig_abs = max|s - s*| / s_max*      <= 1e-5
  resid   = ||A - U S V^T||_F/||A||_F <= 1e-5
  orth    = ||Q^T Q - I||_F / sqrt(k) <= 1e-5
The FP64 references are computed on the FP32-rounded input.
"""
import numpy as np
import pytest

from conftest import golden, golden_names, graded

pytestmark = pytest.mark.gpu

TOL = 1e-5
BASE_MODES = ["plain", "blocked"]


def tc_modes(lib):
    return [m for m in ("tf32x6", "tf32x3", "bf16x3") if _mode_available(lib, m)]


_avail = {}


def _mode_available(lib, mode):
    if mode not in _avail:
        import torch
        try:
            lib.svd_device(torch.ones((4, 4), device="cuda"), mode=mode)
            _avail[mode] = True
        except lib.DdcsvdError as e:
            assert e.status == 8, e  # only "unsupported" may mark a mode unavailable
            _avail[mode] = False
    return _avail[mode]


def run(lib, torch, A, mode):
    s, U, V = lib.svd_device(torch.from_numpy(np.asarray(A, dtype=np.float32)).cuda(), mode=mode)
    torch.cuda.synchronize()
    return s.double().cpu().numpy(), U.double().cpu().numpy(), V.double().cpu().numpy()


def check_metrics(orc, A, s, U, V, tol=TOL, sig_true=None):
    A64 = np.asarray(A, dtype=np.float32).astype(np.float64)
    if sig_true is None:
        sig_true = np.linalg.svd(A64, compute_uv=False)
    met = orc.metrics(A64, s, U, V, sig_true)
    assert np.all(np.diff(s) >= 0), "singular values must come out ascending"
    assert met["sig_abs"] <= tol and met["resid"] <= tol, met
    assert met["orth_u"] <= tol and met["orth_v"] <= tol, met
    return met


# ------------------------------------------------------------------ end to end
SHAPES = [(1, 1), (2, 2), (3, 3), (2, 1), (1, 3), (5, 3), (3, 5), (17, 17), (33, 20), (64, 64), (100, 37),
          (20, 33), (128, 96), (257, 129), (512, 256)]


@pytest.mark.parametrize("mode", BASE_MODES)
@pytest.mark.parametrize("m,n", SHAPES)
def test_svd_uniform(lib, cuda, orc, mode, m, n):
    rng = np.random.default_rng(m * 7919 + n)
    A = rng.uniform(-1, 1, (m, n)).astype(np.float32)
    s, U, V = run(lib, cuda, A, mode)
    check_metrics(orc, A, s, U, V)


@pytest.mark.parametrize("m,n", [(64, 64), (257, 129), (512, 256), (300, 1000)])
def test_svd_tensor_core_modes(lib, cuda, orc, m, n):
    modes = tc_modes(lib)
    if not modes:
        pytest.skip("tensor-core modes not built")
    rng = np.random.default_rng(m + n)
    A = rng.uniform(-1, 1, (m, n)).astype(np.float32)
    for mode in modes:
        s, U, V = run(lib, cuda, A, mode)
        check_metrics(orc, A, s, U, V)


@pytest.mark.parametrize("mode", BASE_MODES)
@pytest.mark.parametrize("kind", ["identity", "zero", "diag_repeated", "rank_deficient", "graded", "block"])
def test_svd_structured(lib, cuda, orc, mode, kind):
    n = 96
    rng = np.random.default_rng(5)
    if kind == "identity":
        A = np.eye(n)
    elif kind == "zero":
        A = np.zeros((n, n))
    elif kind == "diag_repeated":
        A = np.diag(np.repeat([3.0, 2.0, 1.0], n // 3))
    elif kind == "rank_deficient":
        A = rng.standard_normal((n, 7)) @ rng.standard_normal((7, n))
    elif kind == "graded":
        A, _ = graded(n)
    else:
        A = np.zeros((n, n))
        A[:40, :40] = rng.standard_normal((40, 40))
        A[40:, 40:] = rng.standard_normal((n - 40, n - 40))
    s, U, V = run(lib, cuda, A, mode)
    A64 = A.astype(np.float32).astype(np.float64)
    st = np.linalg.svd(A64, compute_uv=False)
    assert np.max(np.abs(np.sort(s) - np.sort(st))) <= TOL * max(st.max(), 1e-30)
    if kind != "zero":
        check_metrics(orc, A, s, U, V)


@pytest.mark.parametrize("mode", BASE_MODES)
def test_svd_graded_1024(lib, cuda, orc, mode):
    A, s_true = graded(1024, seed=1)
    s, U, V = run(lib, cuda, A, mode)
    check_metrics(orc, A, s, U, V)


@pytest.mark.parametrize("mode", BASE_MODES)
@pytest.mark.parametrize("kind", ["orthogonal", "two_values", "near_repeated"])
def test_svd_rotated_clusters(lib, cuda, orc, mode, kind):
    """Repeated and nearly repeated singular values behind random rotations, so
    that no zero appears in A: the FP32 bidiagonal carries superdiagonal
    entries at rounding level, which split off at the bidiagonal's own
    accuracy and leave every cluster member in a block of its own."""
    rng = np.random.default_rng(17)
    m, n = {"orthogonal": (600, 600), "two_values": (700, 520), "near_repeated": (640, 480)}[kind]
    if kind == "orthogonal":
        sig = np.ones(n)
    elif kind == "two_values":
        sig = np.repeat([2.0, 1.0], n // 2)
    else:
        sig = np.repeat([3.0, 1.0, 0.25], n // 3) * (1 + 1e-6 * rng.standard_normal(n))
    Q1, _ = np.linalg.qr(rng.standard_normal((m, n)))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = ((Q1 * sig) @ Q2.T).astype(np.float32)
    s, U, V = run(lib, cuda, A, mode)
    check_metrics(orc, A, s, U, V)


def test_svd_matches_oracle_vectors(lib, cuda, orc):
    """Per-vector agreement with the FP64 oracle (up to sign) where sigma is well separated."""
    rng = np.random.default_rng(21)
    A = rng.uniform(-1, 1, (200, 120)).astype(np.float32)
    s, U, V = run(lib, cuda, A, "blocked")
    so, Uo, Vo = orc.svd(A.astype(np.float64))
    assert np.max(np.abs(s - so)) <= 1e-5 * so.max()
    gaps = np.diff(so)
    gap = np.minimum(np.r_[np.inf, gaps], np.r_[gaps, np.inf]) / so.max()
    for k in np.nonzero(gap > 1e-3)[0]:
        assert abs(abs(U[:, k] @ Uo[:, k]) - 1) < 1e-4
        assert abs(abs(V[:, k] @ Vo[:, k]) - 1) < 1e-4


def test_deterministic(lib, cuda):
    rng = np.random.default_rng(3)
    A = rng.uniform(-1, 1, (300, 200)).astype(np.float32)
    r1 = run(lib, cuda, A, "blocked")
    r2 = run(lib, cuda, A, "blocked")
    for a, b in zip(r1, r2):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("mode", ["blocked", "tf32x6"])
@pytest.mark.parametrize("scale", [2.0 ** 60, 2.0 ** -60, 1e30, 1e-30])
def test_svd_extreme_magnitudes(lib, cuda, orc, mode, scale):
    """Inputs far outside [2^-40, 2^40]: the blocked path scales by a power of
    two before its FP32 compensated norms and scales d, e back; sigma must
    follow the input scale and the vectors must be those of the unscaled input."""
    if not _mode_available(lib, mode):
        pytest.skip(f"{mode} unavailable")
    rng = np.random.default_rng(11)
    A = rng.uniform(-1, 1, (200, 120)).astype(np.float32)
    As = (A.astype(np.float64) * scale).astype(np.float32)
    s, U, V = run(lib, cuda, As, mode)
    assert np.all(np.isfinite(s)) and np.all(np.isfinite(U)) and np.all(np.isfinite(V))
    check_metrics(orc, As.astype(np.float64) / scale, s / scale, U, V)


@pytest.mark.parametrize("m,n", [(3000, 2500), (6000, 700)])
def test_svd_large_shapes(lib, cuda, orc, m, n):
    """Sizes beyond the other tests: several thousand rows, many panels, and a
    tall shape whose row blocks per CTA exceed one warp's width."""
    mode = "tf32x6" if _mode_available(lib, "tf32x6") else "blocked"
    rng = np.random.default_rng(m + n)
    A = rng.uniform(-1, 1, (m, n)).astype(np.float32)
    s, U, V = run(lib, cuda, A, mode)
    check_metrics(orc, A, s, U, V)


@pytest.mark.parametrize("m,n,kind", [(600, 256, "uniform"), (1200, 200, "graded"), (256, 700, "uniform"),
                                      (2048, 130, "rank_deficient"), (1001, 300, "uniform"), (4100, 1030, "graded"),
                                      (40000, 160, "uniform")])
def test_svd_tall_qr_path(lib, cuda, orc, m, n, kind):
    """m >= 2n (or n >= 2m) in the tensor-core modes goes through Householder
    QR, the SVD of R and U = Q [U_R; 0].  QR works in 128-column super-blocks
    of 32-column panels: 200, 300 and 1030 columns end in partial super-blocks
    and partial panels; 1001 rows are not a multiple of 4; 40000 rows put 264
    rows in each CTA of the panel kernel."""
    if not _mode_available(lib, "tf32x6"):
        pytest.skip("tf32x6 unavailable")
    rng = np.random.default_rng(m + 7 * n)
    if kind == "graded":
        A = graded(n, seed=3, m=m)[0].astype(np.float32)
    elif kind == "rank_deficient":
        A = (rng.uniform(-1, 1, (m, 40)) @ rng.uniform(-1, 1, (40, n))).astype(np.float32)
    else:
        A = rng.uniform(-1, 1, (m, n)).astype(np.float32)
    h = lib.Handle()
    h.tuning = {"tall_qr": 1}  # these shapes are below the automatic size threshold
    s, U, V = lib.svd_device(cuda.from_numpy(A).cuda(), mode="tf32x6", handle=h)
    cuda.cuda.synchronize()
    check_metrics(orc, A, s.double().cpu().numpy(), U.double().cpu().numpy(), V.double().cpu().numpy())


@pytest.mark.parametrize("fused", [0, 1])
@pytest.mark.parametrize("m,n", [(1023, 517), (2050, 2050), (8200, 100), (40001, 96)])
def test_panel_one_pass_and_two_gemv_forms(lib, cuda, orc, fused, m, n):
    """The panel kernel's one-read form (knob panel_fused = 1, the default up to
    8192 rows) and its two-GEMV form meet the same bounds.  Row counts that are
    not multiples of 4 exercise the ragged last float4; with 8200 rows the first
    panel runs the two-GEMV form and the later ones the one-read form.  With
    40001 rows the staged column no longer fits shared memory beside the panel
    blocks, and y = A^T u reads it from global memory (both knob settings)."""
    if fused == 0 and m > 10000:
        pytest.skip("the same two-GEMV form as the fused setting at this size")
    mode = "tf32x6" if _mode_available(lib, "tf32x6") else "blocked"
    rng = np.random.default_rng(m * 13 + n + fused)
    A = rng.uniform(-1, 1, (m, n)).astype(np.float32)
    h = lib.Handle()
    h.tuning = {"panel_fused": fused, "tall_qr": 0, "panel_tail": 0}
    s, U, V = lib.svd_device(cuda.from_numpy(A).cuda(), mode=mode, handle=h)
    cuda.cuda.synchronize()
    check_metrics(orc, A, s.double().cpu().numpy(), U.double().cpu().numpy(), V.double().cpu().numpy())


@pytest.mark.parametrize("m,n,kind", [(100, 37, "uniform"), (512, 256, "uniform"), (2050, 2050, "uniform"),
                                      (3000, 40, "uniform"), (900, 900, "graded"), (1023, 1001, "uniform")])
def test_bidiag_cluster_tail(lib, cuda, orc, m, n, kind):
    """The last columns on one thread-block cluster (knob panel_tail: at most
    that many columns, default 512) against the panel kernel alone (0): with
    4096 every column that fits the cluster goes there (all of the smaller
    shapes, the last 898 of 2050 x 2050), with 512 the hand-over is at
    n - 512 where n > 512; all must meet the bounds and agree on sigma."""
    mode = "tf32x6" if _mode_available(lib, "tf32x6") else "blocked"
    rng = np.random.default_rng(m * 3 + n)
    A = graded(n, seed=4, m=m)[0].astype(np.float32) if kind == "graded" else \
        rng.uniform(-1, 1, (m, n)).astype(np.float32)
    outs = []
    for tail in (4096, 512, 0):
        h = lib.Handle()
        h.tuning = {"panel_tail": tail, "tall_qr": 0}
        s, U, V = lib.svd_device(cuda.from_numpy(A).cuda(), mode=mode, handle=h)
        cuda.cuda.synchronize()
        s, U, V = s.double().cpu().numpy(), U.double().cpu().numpy(), V.double().cpu().numpy()
        check_metrics(orc, A, s, U, V)
        outs.append(s)
    for o in outs[:2]:
        assert np.max(np.abs(o - outs[2])) <= TOL * outs[2].max()


@pytest.mark.parametrize("mode", ["blocked", "tf32x6"])
def test_bidiag_caller_padding_not_used(lib, cuda, mode):
    """Rows m .. lda-1 of a caller's buffer may hold anything: with NaN there the
    bidiagonal is bit-identical to the zero-padded run (m = 301, lda = 320)."""
    if mode == "tf32x6" and not _mode_available(lib, mode):
        pytest.skip("tf32x6 unavailable")
    torch = cuda
    m, n = 301, 150
    ldw = 320
    A = torch.from_numpy(np.random.default_rng(5).uniform(-1, 1, (m, n)).astype(np.float32)).cuda()
    h = lib.Handle()
    outs = []
    for fill in (0.0, float("nan")):
        W = torch.full((n, ldw), fill, dtype=torch.float32, device="cuda")
        W[:, :m] = A.t()
        d, e, tq, tp = (torch.zeros(n, dtype=torch.float32, device="cuda") for _ in range(4))
        lib.check(lib.load().ddcsvd_bidiag_f32_device(h.ptr, m, n, W.data_ptr(), ldw, d.data_ptr(), e.data_ptr(),
                                                      tq.data_ptr(), tp.data_ptr(), lib._mode(mode)), "bidiag")
        torch.cuda.synchronize()
        outs.append((d.cpu().numpy(), e[: n - 1].cpu().numpy()))
    assert np.all(np.isfinite(outs[1][0])) and np.all(np.isfinite(outs[1][1]))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def _form_factors_numpy(A_mod, left):
    """The reference's form_u_par / form_v_par loops (bidiag_par.c:877-988), restated in numpy."""
    m, n = A_mod.shape
    mn = min(m, n)
    if left:
        Q = np.eye(m)
        for i in range(m):
            for j in range(min(i, mn - 1), -1, -1):
                v = A_mod[j:, j]
                Q[j:, i] -= 2.0 * v * (v @ Q[j:, i])
        return Q
    nref = mn if m < n else mn - 1
    Q = np.eye(n)
    for i in range(n):
        for j in range(min(i - 1, nref - 1), -1, -1):
            v = A_mod[j, j + 1:]
            Q[j + 1:, i] -= 2.0 * v * (v @ Q[j + 1:, i])
    return Q


@pytest.mark.parametrize("m,n", [(40, 40), (90, 57), (257, 130), (57, 90), (1, 6), (130, 131)])
def test_form_factors_dropin(lib, cuda, m, n):
    """form_u_par / form_v_par on bidiag_par's reflectors: the reference's loops
    (numpy restatement) to FP64 accuracy; orthogonality and A = U [B; 0] V^T
    to the FP32 level of the bidiagonalisation."""
    rng = np.random.default_rng(m * 31 + n)
    A = rng.uniform(-1, 1, (m, n))
    A_mod, al, be = lib.bidiag_par(A)
    U = lib.form_u_par(A_mod)
    V = lib.form_v_par(A_mod)
    assert np.abs(U - _form_factors_numpy(A_mod, True)).max() <= 1e-12
    assert np.abs(V - _form_factors_numpy(A_mod, False)).max() <= 1e-12
    # the reflectors come from the FP32 bidiagonalisation (||v|| = 1 to FP32):
    # orthogonal to the FP32 level
    assert np.linalg.norm(U.T @ U - np.eye(m)) / m ** 0.5 <= TOL
    assert np.linalg.norm(V.T @ V - np.eye(n)) / n ** 0.5 <= TOL
    B = _bidiagonal(m, n, al, be)
    A32 = A.astype(np.float32).astype(np.float64)
    assert np.linalg.norm(U @ B @ V.T - A32) / np.linalg.norm(A32) <= 1e-5


@pytest.mark.parametrize("shape,bad,mode,tall_qr", [((16, 8), np.nan, "blocked", 0),
                                                    ((300, 130), np.inf, "tf32x3", 1),
                                                    ((40, 200), -np.inf, "tf32x3", 0)])
def test_nonfinite_input_fails_loudly(lib, cuda, shape, bad, mode, tall_qr):
    """A NaN or Inf entry is found while the input is copied into the working
    matrix (the direct path, the QR-first path and a wide input alike)."""
    if mode != "blocked" and not _mode_available(lib, mode):
        pytest.skip(f"{mode} unavailable")
    A = np.ones(shape, dtype=np.float32)
    A[shape[0] // 2, shape[1] - 1] = bad
    h = lib.Handle()
    h.tuning = {"tall_qr": tall_qr}
    with pytest.raises(lib.DdcsvdError) as ei:
        lib.svd_device(cuda.from_numpy(A).cuda(), mode=mode, handle=h)
    assert ei.value.status == 7
    s, U, V = lib.svd_device(cuda.from_numpy(np.eye(8, dtype=np.float32)).cuda(), mode=mode, handle=h)
    assert np.allclose(s.cpu().numpy(), 1.0)  # handle still usable


# ------------------------------------------------------------------ stage parity
@pytest.mark.parametrize("mode", BASE_MODES)
@pytest.mark.parametrize("m,n", [(8, 8), (33, 20), (100, 100), (260, 130), (513, 300)])
def test_bidiag_stage_vs_oracle(lib, cuda, orc, mode, m, n):
    rng = np.random.default_rng(m * 31 + n)
    A = rng.uniform(-1, 1, (m, n)).astype(np.float32)
    W, d, e, tq, tp = lib.bidiag_device(cuda.from_numpy(A).cuda(), mode=mode)
    _, al, be = orc.bidiag(A.astype(np.float64))
    d = d.double().cpu().numpy()
    e = e.double().cpu().numpy()
    # same reflector sign convention as the reference: entries agree, not only |entries|.
    # Individual bidiagonal entries are not well conditioned; bound by FP32 backward error.
    tol = 1e-5 * np.sqrt(n) * np.linalg.norm(A, 2)
    assert np.max(np.abs(d - al)) <= tol
    assert np.max(np.abs(e - be)) <= tol
    # the singular values of the bidiagonal are well conditioned
    B = np.diag(d) + np.diag(e, 1)
    Bo = np.diag(al) + np.diag(be, 1)
    assert np.max(np.abs(np.linalg.svd(B, compute_uv=False) - np.linalg.svd(Bo, compute_uv=False))) <= \
        2e-6 * np.linalg.norm(A, 2)


def _reflector_factors(A_r, m, n):
    """Q, P from reflectors stored the reference's way (bidiag_par.c:63-68):
    left reflector i in A_r[i:, i], right reflector i in A_r[i, i+1:], H = I - 2 v v^T.
    A wide matrix (m < n) has m left reflectors (the last one zero: no
    reflection) and m right ones (bidiag.c:130-155)."""
    Q, P = np.eye(m), np.eye(n)
    for i in range(min(m, n)):
        v = np.zeros(m)
        v[i:] = A_r[i:, i]
        Q = Q - 2.0 * np.outer(Q @ v, v)
    for i in range(m if m < n else max(n - 2, 0)):
        v = np.zeros(n)
        v[i + 1:] = A_r[i, i + 1:]
        P = P - 2.0 * np.outer(P @ v, v)
    return Q, P


def _bidiagonal(m, n, al, be):
    """The m x n upper bidiagonal: alpha on the diagonal, beta above it
    (min(m, n) - 1 entries when m >= n, m when m < n)."""
    B = np.zeros((m, n))
    k = min(m, n)
    B[np.arange(k), np.arange(k)] = al
    nb = len(be)
    B[np.arange(nb), np.arange(1, nb + 1)] = be
    return B


@pytest.mark.parametrize("name", golden_names("bidiag_"))
def test_bidiag_par_dropin_vs_reference(lib, cuda, name):
    """Square, tall and wide matrices against the reference's own outputs;
    wide ones reduce to the m x (m+1) upper bidiagonal with the reference's
    last-row edge case."""
    g = golden(name)
    A = g["A"]
    m, n = A.shape
    A_r, al, be = lib.bidiag_par(A)
    assert al.shape == g["alpha"].shape and be.shape == g["beta"].shape
    scale = np.linalg.norm(A, 2)
    tol = 1e-5 * np.sqrt(max(m, n)) * scale
    assert np.max(np.abs(al - g["alpha"])) <= tol
    if len(be):
        assert np.max(np.abs(be - g["beta"])) <= tol
    # the exported reflectors (reference storage) reproduce A = Q B P^T
    Q, P = _reflector_factors(A_r, m, n)
    B = _bidiagonal(m, n, al, be)
    assert np.linalg.norm(A - Q @ B @ P.T) <= 1e-5 * np.linalg.norm(A)
    assert np.linalg.norm(Q.T @ Q - np.eye(m)) <= 1e-5 * np.sqrt(m)
    # and agree with the reference's FP64 reflectors to FP32 conditioning
    ok = np.isfinite(g["A_refl"])
    assert np.max(np.abs(A_r[ok] - g["A_refl"][ok])) <= 5e-3


@pytest.mark.parametrize("N", [1, 2, 3, 4, 7, 64, 300, 1000])
@pytest.mark.parametrize("rect", [False, True])
def test_dc_stage_vs_oracle(lib, cuda, orc, N, rect):
    rng = np.random.default_rng(N + 100 * rect)
    b1 = rng.uniform(0.2, 2.0, N)
    b2 = rng.uniform(0.2, 2.0, N)
    if not rect:
        b2[-1] = 0.0
    s = lib.bdsdc_sigma_device(cuda.from_numpy(b1).cuda(), cuda.from_numpy(b2).cuda()).cpu().numpy()
    so = orc.dc_sigma(b1, b2)
    assert np.max(np.abs(s - so)) <= 1e-13 * so.max()
    assert np.max(np.abs(s - so) / so) <= 1e-11


@pytest.mark.parametrize("kind", ["graded", "split", "repeated", "tiny_z"])
def test_dc_stage_hard_cases(lib, cuda, orc, kind):
    N = 257
    rng = np.random.default_rng(9)
    b1 = rng.uniform(0.5, 1.5, N)
    b2 = rng.uniform(0.5, 1.5, N)
    b2[-1] = 0.0
    if kind == "graded":
        b1 *= 10.0 ** (-6 * np.arange(N) / N)
        b2 *= 10.0 ** (-6 * np.arange(N) / N)
    elif kind == "split":
        b2[[10, 11, 100, 200]] = 0.0
    elif kind == "repeated":
        b1[:] = 1.0
        b2[::2] = 0.0
    else:
        b2[50:60] = 1e-18
    s = lib.bdsdc_sigma_device(cuda.from_numpy(b1).cuda(), cuda.from_numpy(b2).cuda()).cpu().numpy()
    so, _, _ = orc.bdsvd(b1, b2)
    B = np.diag(b1) + np.diag(b2[:-1], 1)
    st = np.sort(np.linalg.svd(B, compute_uv=False))
    assert np.max(np.abs(s - st)) <= 1e-12 * st.max()
    assert np.max(np.abs(s - so)) <= 1e-12 * st.max()


@pytest.mark.parametrize("N", [1, 2, 5, 64, 500])
@pytest.mark.parametrize("kind", ["uniform", "graded", "split"])
def test_vector_stage_vs_oracle(lib, cuda, orc, N, kind):
    rng = np.random.default_rng(N * 3 + len(kind))
    a = rng.uniform(0.5, 1.5, N)
    b = rng.uniform(0.5, 1.5, max(N - 1, 0))
    if kind == "graded":
        a *= 10.0 ** (-6 * np.arange(N) / max(N, 1))
        b *= 10.0 ** (-6 * np.arange(1, N) / max(N, 1))
    elif kind == "split" and N > 4:
        b[N // 2] = 0.0
    so, Xo, b_split = orc.bdsvd(a, b)
    T = cuda
    s_gpu = lib.bdsdc_sigma_device(T.from_numpy(a).cuda(), T.from_numpy(np.r_[b, 0.0]).cuda())
    X, Y = lib.bdvec_device(T.from_numpy(a).cuda(), T.from_numpy(np.r_[b, 0.0]).cuda(), s_gpu)
    X = X.double().cpu().numpy()
    Y = Y.double().cpu().numpy()
    k = N
    assert np.linalg.norm(X.T @ X - np.eye(k)) / np.sqrt(k) <= 1e-6
    assert np.linalg.norm(Y.T @ Y - np.eye(k)) / np.sqrt(k) <= 1e-6
    B = np.diag(a) + (np.diag(b_split, 1) if N > 1 else 0)
    R = B @ X - Y * so
    assert np.linalg.norm(R) <= 1e-6 * np.linalg.norm(B) * np.sqrt(k)
    for j in range(N):  # per vector, against the oracle (FP32 output)
        assert abs(abs(X[:, j] @ Xo[:, j]) - 1) <= 1e-6


def _clustered_bidiagonal(kind):
    """Unreduced bidiagonals (every superdiagonal entry 1, nothing splits) whose
    singular values coincide to working precision: large diagonal entries at
    both ends give pairs, three peaks give triples."""
    if kind in ("pairs41", "pairs201"):
        h = 20 if kind == "pairs41" else 100
        a = np.abs(np.arange(2 * h + 1) - h) + 1.0
    else:
        P = 24
        a = np.abs((np.arange(3 * P + 1) % P) - P / 2) + 1.0
    return a, np.ones(len(a) - 1)


@pytest.mark.parametrize("kind", ["pairs41", "pairs201", "triples73"])
def test_vector_stage_clusters(lib, cuda, orc, kind):
    """Singular values equal to working precision inside one unreduced block:
    the twisted solve alone returns the same vector for equal values (the FP64
    oracle, which follows the reference's method, is far from orthogonal
    here); the cluster step must give orthonormal X and Y with B X = Y S."""
    a, b = _clustered_bidiagonal(kind)
    N = len(a)
    B = np.diag(a) + np.diag(b, 1)
    st = np.sort(np.linalg.svd(B, compute_uv=False))
    assert np.sum(np.diff(st) <= 1e-10 * st.max()) >= 10  # the case really has clusters
    _, Xo, _ = orc.bdsvd(a, b)
    assert np.linalg.norm(Xo.T @ Xo - np.eye(N)) / np.sqrt(N) > 1e-2  # and the plain method fails on it
    T = cuda
    b2 = np.r_[b, 0.0]
    s = lib.bdsdc_sigma_device(T.from_numpy(a).cuda(), T.from_numpy(b2).cuda())
    X, Y = lib.bdvec_device(T.from_numpy(a).cuda(), T.from_numpy(b2).cuda(), s)
    s = s.cpu().numpy()
    X = X.double().cpu().numpy()
    Y = Y.double().cpu().numpy()
    assert np.max(np.abs(s - st)) <= 1e-12 * st.max()
    assert np.linalg.norm(X.T @ X - np.eye(N)) / np.sqrt(N) <= 1e-6
    assert np.linalg.norm(Y.T @ Y - np.eye(N)) / np.sqrt(N) <= 1e-6
    assert np.linalg.norm(B @ X - Y * s) <= 1e-6 * np.linalg.norm(B) * np.sqrt(N)


# ------------------------------------------------------------------ drop-ins vs the reference
@pytest.mark.parametrize("name", golden_names("svd_"))
def test_svd_gpu_dropin_vs_reference(lib, cuda, orc, name):
    g = golden(name)
    s, U, V = lib.svd_gpu(g["A"])
    smax = g["sigma_lapack"].max()
    assert np.all(np.diff(s) >= 0)
    assert np.max(np.abs(s - g["sigma_lapack"])) <= 1e-5 * smax  # vs LAPACK (FP64)
    if np.all(np.isfinite(g["sigma"])):
        assert np.max(np.abs(s - g["sigma"])) <= 1e-4 * smax     # vs the reference, to its accuracy
    check_metrics(orc, g["A"], s, U, V, sig_true=g["sigma_lapack"])
    gaps = np.diff(s)
    gap = np.minimum(np.r_[np.inf, gaps], np.r_[gaps, np.inf]) / smax
    Ur = g["U"].astype(np.float64)
    for k in range(len(s)):
        if gap[k] > 1e-2 and np.all(np.isfinite(Ur[:, k])):
            assert abs(abs(U[:, k] @ Ur[:, k]) / np.linalg.norm(Ur[:, k]) - 1) < 1e-3


def test_void_dropin_signature(lib, cuda):
    rng = np.random.default_rng(1)
    A = rng.uniform(1, 4, (40, 40))
    s, U, V = lib.svd_gpu_void(A)
    assert np.allclose(np.sort(s), np.sort(np.linalg.svd(A, compute_uv=False)), rtol=0, atol=1e-5 * 40 * 2.5)


def test_host_f32_api(lib, cuda, orc):
    rng = np.random.default_rng(2)
    A = rng.uniform(-1, 1, (150, 90)).astype(np.float32)
    s, U, V = lib.svd(A)
    check_metrics(orc, A, s.astype(np.float64), U.astype(np.float64), V.astype(np.float64))


@pytest.mark.parametrize("mode,m,n,tall_qr", [("plain", 60000, 8, 0), ("tf32x6", 262144, 128, 1),
                                              ("tf32x6", 262144, 128, 0)])
def test_row_limits_report_arg(lib, cuda, mode, m, n, tall_qr):
    """Beyond the rows that the panel kernels hold in shared memory (plain
    FP32 path: the whole column, ~56K rows; QR and direct panels: a 1/152
    slice of the rows times 33 floats, ~250K rows) a call fails with
    DDCSVD_ERR_ARG and a message naming the limit, and the handle still
    gives correct results afterwards."""
    if mode == "tf32x6" and not _mode_available(lib, mode):
        pytest.skip("tf32x6 unavailable")
    A = cuda.zeros((m, n), dtype=cuda.float32, device="cuda")
    A[:n, :n] = cuda.eye(n, device="cuda")
    h = lib.Handle()
    h.tuning = {"tall_qr": tall_qr}
    with pytest.raises(lib.DdcsvdError) as ei:
        lib.svd_device(A, mode=mode, handle=h)
    assert ei.value.status == 1
    assert "too many rows" in str(ei.value)
    cuda.cuda.synchronize()
    B = np.random.default_rng(9).uniform(-1, 1, (300, 200)).astype(np.float32)
    s, U, V = lib.svd_device(cuda.from_numpy(B).cuda(), mode=mode, handle=h)
    st = np.sort(np.linalg.svd(B.astype(np.float64), compute_uv=False))
    assert np.max(np.abs(s.double().cpu().numpy() - st)) <= TOL * st[-1]


@pytest.mark.parametrize("stream_kind", ["legacy", "user"])
def test_side_stream_overlap_keeps_stream_order(lib, cuda, orc, stream_kind):
    """The tensor-core modes prepare the back-transformation on the handle's
    second stream while stages 2-4 run and join it before stage 5.  On the
    legacy default stream (a null stream handle) and on a user stream alike,
    every later call of the handle must again run on the caller's stream:
    a GEMM right after the SVD reads inputs that torch has only just queued
    on that stream."""
    if not _mode_available(lib, "tf32x6"):
        pytest.skip("tf32x6 unavailable")
    torch = cuda
    s = torch.cuda.current_stream() if stream_kind == "legacy" else torch.cuda.Stream()
    with torch.cuda.stream(s):
        h = lib.Handle(stream=s)
        rng = np.random.default_rng(31)
        A = rng.uniform(-1, 1, (700, 500)).astype(np.float32)
        sv, U, V = lib.svd_device(torch.from_numpy(A).cuda(), mode="tf32x6", handle=h)
        g = torch.Generator(device="cuda").manual_seed(5)
        X = torch.rand((256, 2048), device="cuda", generator=g) * 2 - 1
        Y = torch.rand((192, 2048), device="cuda", generator=g) * 2 - 1
        C = lib.gemm_nt_device(X, Y, mode="tf32x6", handle=h)
        ref = X.double() @ Y.double().T
        err = float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref))
        res = (sv.double().cpu().numpy(), U.double().cpu().numpy(), V.double().cpu().numpy())
    s.synchronize()
    assert err <= 1e-6, err
    check_metrics(orc, A, *res)


def test_host_f32_api_on_handle(lib, cuda, orc):
    """ddcsvd_svd_f32_host: host buffers on a handle (its knobs and stream);
    a strided host layout (ld larger than the rows) for every matrix."""
    import ctypes
    if not _mode_available(lib, "tf32x3"):
        pytest.skip("tf32x3 unavailable")
    rng = np.random.default_rng(41)
    m, n = 333, 201
    A = rng.uniform(-1, 1, (m, n)).astype(np.float32)
    lda, ldu, ldv = m + 3, m + 5, n + 2
    Ab = np.zeros((n, lda), dtype=np.float32)
    Ab[:, :m] = A.T
    s = np.zeros(n, dtype=np.float32)
    Ub = np.zeros((n, ldu), dtype=np.float32)
    Vb = np.zeros((n, ldv), dtype=np.float32)
    h = lib.Handle()
    h.tuning = {"splitk_max": 2}
    addr = lambda x: x.ctypes.data
    rc = lib.load().ddcsvd_svd_f32_host(h.ptr, m, n, addr(Ab), lda, addr(s), addr(Ub), ldu, addr(Vb), ldv,
                                        lib.MODES["tf32x3"])
    lib.check(rc, "ddcsvd_svd_f32_host")
    check_metrics(orc, A, s.astype(np.float64), Ub[:, :m].T.astype(np.float64), Vb[:, :n].T.astype(np.float64))
