"""The hand-written SVD adjoint (ddcsvd_svd_backward_*) against central finite
differences in FP64 and against torch.linalg.svd's gradient.

Configuration shape: A = Q1 diag(sigma) Q2^T with Haar Q1, Q2 and
sigma_i = 1 + i/64 (distinct, gaps >= 1/64); loss = w^T s + <G_U, U> + <G_V, V>.
The forward for the finite differences is LAPACK in FP64 with a fixed sign
gauge (each right vector's largest entry positive), under which U and V are
smooth functions of A."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_problem(rng, m=128, n=64):
    Q1, R1 = np.linalg.qr(rng.standard_normal((m, n)))
    Q1 *= np.sign(np.diag(R1))
    Q2, R2 = np.linalg.qr(rng.standard_normal((n, n)))
    Q2 *= np.sign(np.diag(R2))
    s = 1.0 + np.arange(n) / 64.0
    return (Q1 * s) @ Q2.T


def gauge_svd(A):
    U, s, Vt = np.linalg.svd(A, full_matrices=False)
    V = Vt.T
    idx = np.argmax(np.abs(V), axis=0)
    sg = np.sign(V[idx, np.arange(V.shape[1])])
    return U * sg, s, V * sg


def loss(A, w, GU, GV):
    U, s, V = gauge_svd(A)
    return w @ s + np.sum(GU * U) + np.sum(GV * V)


def adjoint_gpu(lib, torch, U, s, V, gU, gs, gV, dtype):
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to("cuda", dtype)  # noqa: E731
    gA = lib.svd_backward_device(t(U)[None], t(s)[None], t(V)[None], t(gU)[None], t(gs)[None], t(gV)[None])
    return gA[0].double().cpu().numpy()


@pytest.mark.parametrize("seed", [4, 5, 6])
def test_adjoint_f64_vs_central_differences(lib, cuda, seed):
    rng = np.random.default_rng(seed)
    A = make_problem(rng)
    w = rng.standard_normal(64)
    GU = rng.standard_normal((128, 64))
    GV = rng.standard_normal((64, 64))
    U, s, V = gauge_svd(A)
    gA = adjoint_gpu(lib, cuda, U, s, V, GU, w, GV, cuda.float64)
    h = 1e-6
    for _ in range(6):
        E = rng.standard_normal(A.shape)
        E /= np.linalg.norm(E)
        fd = (loss(A + h * E, w, GU, GV) - loss(A - h * E, w, GU, GV)) / (2 * h)
        an = np.sum(gA * E)
        assert abs(fd - an) <= 1e-6 * max(abs(fd), np.linalg.norm(gA) * 1e-3), (fd, an)


def test_adjoint_matches_torch_autograd(lib, cuda):
    torch = cuda
    rng = np.random.default_rng(7)
    for dtype, tol in ((torch.float64, 1e-9), (torch.float32, 2e-4)):
        A = make_problem(rng)
        w = rng.standard_normal(64)
        GU = rng.standard_normal((128, 64))
        GV = rng.standard_normal((64, 64))
        At = torch.tensor(A, dtype=torch.float64, requires_grad=True)
        U, s, Vh = torch.linalg.svd(At, full_matrices=False)
        V = Vh.T
        L = (torch.tensor(w) * s).sum() + (torch.tensor(GU) * U).sum() + (torch.tensor(GV) * V).sum()
        L.backward()
        ref = At.grad.numpy()
        got = adjoint_gpu(lib, torch, U.detach().numpy(), s.detach().numpy(), V.detach().numpy(), GU, w, GV, dtype)
        assert np.linalg.norm(got - ref) <= tol * np.linalg.norm(ref)


def test_adjoint_batch_and_null_gradients(lib, cuda):
    torch = cuda
    rng = np.random.default_rng(8)
    B = 5
    As = [make_problem(rng) for _ in range(B)]
    trip = [gauge_svd(A) for A in As]
    Us = torch.tensor(np.stack([t[0] for t in trip]), device="cuda")
    Ss = torch.tensor(np.stack([t[1] for t in trip]), device="cuda")
    Vs = torch.tensor(np.stack([t[2] for t in trip]), device="cuda")
    gs = torch.tensor(rng.standard_normal((B, 64)), device="cuda")
    gA = lib.svd_backward_device(Us, Ss, Vs, None, gs, None).cpu().numpy()
    for b in range(B):  # d(w^T s)/dA = U diag(w) V^T
        U, s, V = trip[b]
        ref = (U * gs[b].cpu().numpy()) @ V.T
        assert np.allclose(gA[b], ref, atol=1e-12)


def test_autograd_function_end_to_end(lib, cuda):
    """Forward through the CUDA SVD, backward through the adjoint kernel (FP32),
    against torch.linalg.svd in FP64 on a sign-invariant loss."""
    torch = cuda
    from ddcsvd.autograd import svd as ddc_svd
    rng = np.random.default_rng(9)
    A = torch.tensor(np.stack([make_problem(rng) for _ in range(4)]), dtype=torch.float32, device="cuda")
    w = torch.tensor(rng.standard_normal(64), dtype=torch.float32, device="cuda")
    g = torch.tensor(rng.standard_normal(128), dtype=torch.float32, device="cuda")

    def f(U, S, V):  # sign-invariant: sum_j w_j s_j + (g^T u_j)^2
        return (S * w.to(S.dtype)).sum() + ((g.to(U.dtype) @ U) ** 2).sum()

    A1 = A.clone().requires_grad_(True)
    U, S, V = ddc_svd(A1)
    # ddcsvd returns ascending sigma; torch descending: reverse w for the comparison
    f(U, S, V).backward()
    A2 = A.double().clone().requires_grad_(True)
    U2, S2, V2h = torch.linalg.svd(A2, full_matrices=False)
    f(U2.flip(-1), S2.flip(-1), V2h.transpose(-1, -2).flip(-1)).backward()
    rel = float(torch.linalg.norm(A1.grad.double() - A2.grad) / torch.linalg.norm(A2.grad))
    assert rel <= 1e-3, rel
