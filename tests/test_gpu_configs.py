"""Parity at the five benchmark configurations themselves (GPU, C ABI).

The reference's own check of a whole SVD is compiled out
(test-whole-svd.c:81-96), so these tests pin the configurations the
pipeline (svd_gpu.c:53-131) is measured on, at their full sizes:

* plain 512 x 256, U[-1, 1] from default_rng(0), FP32 entries: against the
  reference's own outputs on that exact input (tests/golden/svd_cfg_512x256,
  produced by the reference's host code compiled from its sources) -- sigma
  to the reference's accuracy (its secular solve stops at |g| <= 1e-5,
  Calculations-Parallel.c:163), U up to sign where sigma is separated; V is
  left out because the reference's V is wrong for m != n (multV's leading
  dimension) -- and against LAPACK in FP64, in every mode;
* 4096 x 4096 graded (sigma_i = 10^(-6 i/4095), Haar factors from QR of
  default_rng(1) Gaussians, FP32 entries), every mode: FP64 residual,
  orthogonality of U and V and the singular values against the known
  spectrum, all <= 1e-5, computed on the GPU;
* 16384 x 8192 thin SVD, N(0, 1) entries from default_rng(2): FP64 residual
  and orthogonality on the GPU in column chunks, <= 1e-5;
* the adjoint on 256 problems of 128 x 64 (sigma_i = 1 + i/64, Haar factors
  from default_rng(4); w, G_U, G_V from default_rng(5)): FP64 against
  central differences (h = 1e-6) to 1e-6 relative, FP64 and FP32 against
  torch.linalg.svd's gradient, and the FP32 forward + adjoint through the
  autograd wrapper on a sign-invariant loss.
"""
import numpy as np
import pytest

from conftest import golden, graded

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _modes(lib, cuda):
    out = ["plain", "blocked"]
    for m in ("tf32x3", "tf32x6"):
        try:
            lib.svd_device(cuda.ones((4, 4), device="cuda"), mode=m)
            out.append(m)
        except lib.DdcsvdError as e:
            assert e.status == 8, e
    return out


def _fp64_metrics(torch, A64, s, U, V, s_true=None):
    """resid, orth_u, orth_v (and sig_abs against s_true) in FP64 on the GPU."""
    s64, U64, V64 = s.double(), U.double(), V.double()
    k = s64.shape[0]
    eye = torch.eye(k, dtype=torch.float64, device=A64.device)
    out = {"resid": float(torch.linalg.norm(A64 - (U64 * s64) @ V64.T) / torch.linalg.norm(A64)),
           "orth_u": float(torch.linalg.norm(U64.T @ U64 - eye) / k ** 0.5),
           "orth_v": float(torch.linalg.norm(V64.T @ V64 - eye) / k ** 0.5)}
    if s_true is not None:
        st = torch.sort(torch.as_tensor(s_true, dtype=torch.float64, device=A64.device)).values
        out["sig_abs"] = float(torch.max(torch.abs(torch.sort(s64).values - st)) / st[-1])
    return out


# ------------------------------------------------------------------ plain 512 x 256
def test_config_plain_512x256_vs_reference_outputs(lib, cuda, orc):
    torch = cuda
    g = golden("svd_cfg_512x256")
    A = g["A"]
    assert A.shape == (512, 256)
    assert np.array_equal(A, np.random.default_rng(0).uniform(-1, 1, (512, 256)).astype(np.float32))
    smax = g["sigma_lapack"].max()
    gaps = np.diff(g["sigma_lapack"])
    gap = np.minimum(np.r_[np.inf, gaps], np.r_[gaps, np.inf]) / smax
    Ur = g["U"].astype(np.float64)
    # columns whose sigma is separated by more than 5e-4 sigma_max (244 of 256 here): the
    # reference's U agrees with the FP64 oracle there to 2e-9 in 1 - |cos|
    sep = [k for k in range(256) if gap[k] > 5e-4]
    assert len(sep) >= 200
    runs = {"svd_gpu": lib.svd_gpu(A)}
    for mode in _modes(lib, cuda):
        s, U, V = lib.svd_device(torch.from_numpy(A.astype(np.float32)).cuda(), mode=mode)
        runs[mode] = tuple(x.double().cpu().numpy() for x in (s, U, V))
    for name, (s, U, V) in runs.items():
        assert np.all(np.diff(s) >= 0), name
        assert np.max(np.abs(s - g["sigma_lapack"])) <= TOL * smax, name     # vs LAPACK (FP64)
        assert np.max(np.abs(s - g["sigma"])) <= 1e-4 * smax, name           # vs the reference, to its accuracy
        met = orc.metrics(A, s, U, V, g["sigma_lapack"])
        assert met["resid"] <= TOL and met["orth_u"] <= TOL and met["orth_v"] <= TOL, (name, met)
        for k in sep:
            assert abs(abs(U[:, k] @ Ur[:, k]) / np.linalg.norm(Ur[:, k]) - 1) < 1e-4, (name, k)


# ------------------------------------------------------------------ 4096^2 graded
@pytest.fixture(scope="module")
def graded4096(cuda):
    A64, s = graded(4096, seed=1)
    A32 = A64.astype(np.float32)
    return cuda.from_numpy(A32).cuda(), s


@pytest.mark.parametrize("mode", ["tf32x6", "tf32x3", "blocked", "plain"])
def test_config_graded_4096(lib, cuda, graded4096, mode):
    torch = cuda
    if mode not in _modes(lib, cuda):
        pytest.skip(f"{mode} not available")
    A, s_true = graded4096
    s, U, V = lib.svd_device(A, mode=mode)
    torch.cuda.synchronize()
    met = _fp64_metrics(torch, A.double(), s, U, V, s_true)
    assert all(v <= TOL for v in met.values()), (mode, met)
    assert bool(torch.all(s[1:] >= s[:-1]))


# ------------------------------------------------------------------ 16384 x 8192 tall
def test_config_tall_16384x8192(lib, cuda):
    torch = cuda
    m, n = 16384, 8192
    A = torch.from_numpy(np.random.default_rng(2).standard_normal((m, n), dtype=np.float32)).cuda()
    mode = "tf32x6" if "tf32x6" in _modes(lib, cuda) else "blocked"
    s, U, V = lib.svd_device(A, mode=mode)
    torch.cuda.synchronize()
    s64, V64 = s.double(), V.double()
    eye = torch.eye(n, dtype=torch.float64, device="cuda")
    # residual and U^T U in column chunks (FP64 on the GPU)
    r2, a2 = 0.0, 0.0
    UtU = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    for r0 in range(0, m, 4096):
        Ub = U[r0:r0 + 4096].double()
        Ab = A[r0:r0 + 4096].double()
        r2 += float(torch.linalg.norm(Ab - (Ub * s64) @ V64.T) ** 2)
        a2 += float(torch.linalg.norm(Ab) ** 2)
        UtU += Ub.T @ Ub
        del Ub, Ab
    resid = (r2 / a2) ** 0.5
    orth_u = float(torch.linalg.norm(UtU - eye) / n ** 0.5)
    orth_v = float(torch.linalg.norm(V64.T @ V64 - eye) / n ** 0.5)
    assert resid <= TOL and orth_u <= TOL and orth_v <= TOL, (resid, orth_u, orth_v)
    assert bool(torch.all(s[1:] >= s[:-1]))
    # Marchenko-Pastur range of the N(0,1) spectrum: sqrt(m) +- sqrt(n)
    assert 0.9 * (m ** 0.5 - n ** 0.5) < float(s[0]) and float(s[-1]) < 1.1 * (m ** 0.5 + n ** 0.5)


# ------------------------------------------------------------------ adjoint, 256 x (128 x 64)
def _adjoint_config():
    rng = np.random.default_rng(4)
    B, m, n = 256, 128, 64
    Q1, R1 = np.linalg.qr(rng.standard_normal((B, m, n)))
    Q1 = Q1 * np.sign(np.diagonal(R1, axis1=1, axis2=2))[:, None, :]
    Q2, R2 = np.linalg.qr(rng.standard_normal((B, n, n)))
    Q2 = Q2 * np.sign(np.diagonal(R2, axis1=1, axis2=2))[:, None, :]
    s = 1.0 + np.arange(n) / 64.0
    A = (Q1 * s) @ Q2.transpose(0, 2, 1)
    r5 = np.random.default_rng(5)
    w = r5.standard_normal((B, n))
    GU = r5.standard_normal((B, m, n))
    GV = r5.standard_normal((B, n, n))
    return A, w, GU, GV


def _gauge_svd(A):
    """Batched LAPACK SVD with a fixed sign gauge (each right vector's largest
    entry positive), under which U and V are smooth functions of A."""
    U, s, Vt = np.linalg.svd(A, full_matrices=False)
    V = Vt.transpose(0, 2, 1)
    idx = np.argmax(np.abs(V), axis=1)
    sg = np.sign(np.take_along_axis(V, idx[:, None, :], axis=1))
    return U * sg, s, V * sg


def _losses(A, w, GU, GV):
    U, s, V = _gauge_svd(A)
    return np.sum(w * s, axis=1) + np.sum(GU * U, axis=(1, 2)) + np.sum(GV * V, axis=(1, 2))


def test_config_adjoint_fp64_vs_central_differences(lib, cuda):
    torch = cuda
    A, w, GU, GV = _adjoint_config()
    U, s, V = _gauge_svd(A)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()  # noqa: E731
    gA = lib.svd_backward_device(t(U), t(s), t(V), t(GU), t(w), t(GV)).cpu().numpy()
    rng = np.random.default_rng(6)
    h = 1e-6
    worst = 0.0
    for _ in range(3):
        E = rng.standard_normal(A.shape)
        E /= np.linalg.norm(E, axis=(1, 2), keepdims=True)
        fd = (_losses(A + h * E, w, GU, GV) - _losses(A - h * E, w, GU, GV)) / (2 * h)
        an = np.sum(gA * E, axis=(1, 2))
        scale = np.maximum(np.abs(fd), 1e-3 * np.linalg.norm(gA, axis=(1, 2)))
        worst = max(worst, float(np.max(np.abs(fd - an) / scale)))
    assert worst <= 1e-6, worst


@pytest.mark.parametrize("dtype,tol", [("float64", 1e-9), ("float32", 2e-4)])
def test_config_adjoint_vs_torch_gradient(lib, cuda, dtype, tol):
    torch = cuda
    A, w, GU, GV = _adjoint_config()
    At = torch.tensor(A, dtype=torch.float64, requires_grad=True)
    U, s, Vh = torch.linalg.svd(At, full_matrices=False)
    V = Vh.transpose(1, 2)
    L = (torch.tensor(w) * s).sum() + (torch.tensor(GU) * U).sum() + (torch.tensor(GV) * V).sum()
    L.backward()
    ref = At.grad.numpy()
    dt = getattr(torch, dtype)
    c = lambda x: x.detach().to("cuda", dt).contiguous()  # noqa: E731
    got = lib.svd_backward_device(c(U), c(s), c(V), c(torch.tensor(GU)), c(torch.tensor(w)),
                                  c(torch.tensor(GV))).double().cpu().numpy()
    rel = np.linalg.norm(got - ref, axis=(1, 2)) / np.linalg.norm(ref, axis=(1, 2))
    assert float(rel.max()) <= tol, float(rel.max())


def test_config_autograd_forward_and_adjoint_fp32(lib, cuda):
    """The CUDA forward (FP32 SVD of all 256 problems) and the FP32 adjoint
    through the autograd wrapper, against torch.linalg.svd in FP64, on a loss
    that does not depend on the vectors' signs."""
    torch = cuda
    from ddcsvd.autograd import svd as ddc_svd
    A, w, GU, _ = _adjoint_config()
    Ad = torch.tensor(A, device="cuda")
    wt = torch.tensor(w, device="cuda")
    g = torch.tensor(GU[:, :, 0], device="cuda")  # one direction per problem

    def f(U, S):
        return (S * wt.to(S.dtype)).sum() + ((g.to(U.dtype)[:, None, :] @ U) ** 2).sum()

    A1 = Ad.float().clone().requires_grad_(True)
    U, S, V = ddc_svd(A1)
    # ascending sigma here, descending in torch: flip torch's to match w
    f(U, S).backward()
    A2 = Ad.clone().requires_grad_(True)
    U2, S2, _ = torch.linalg.svd(A2, full_matrices=False)
    f(U2.flip(-1), S2.flip(-1)).backward()
    rel = torch.linalg.norm(A1.grad.double() - A2.grad, dim=(1, 2)) / torch.linalg.norm(A2.grad, dim=(1, 2))
    assert float(rel.max()) <= 1e-3, float(rel.max())
