"""GEMM back ends (CUDA-core FP32, tcgen05 split TF32) against FP64 products."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("K", [8, 64, 512, 4096])
def test_gemm_backends_accuracy(lib, cuda, K):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(K)
    M, N = 256, 192
    A = torch.rand((M, K), device="cuda", generator=g) * 2 - 1
    B = torch.rand((N, K), device="cuda", generator=g) * 2 - 1
    ref = A.double() @ B.double().T
    errs = {}
    for mode in ("blocked", "tf32x3", "tf32x6"):
        C = lib.gemm_nt_device(A, B, mode=mode)
        errs[mode] = float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref))
    print(f"K={K} rel err", {k: f"{v:.2e}" for k, v in errs.items()})
    # FP32-level: within a small factor of the CUDA-core FMA result
    assert errs["blocked"] <= 2e-6
    assert errs["tf32x6"] <= max(3 * errs["blocked"], 2e-7)
    assert errs["tf32x3"] <= 5e-6


def test_gemm_update_form(lib, cuda):
    """C = beta C + alpha A B^T with a nonzero C, ragged sizes (TMA zero fill)."""
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(1)
    M, N, K = 300, 130, 72  # K not a multiple of 32 (TMA zero fill); rows stay 16-byte aligned
    A = torch.rand((M, K), device="cuda", generator=g) * 2 - 1
    B = torch.rand((N, K), device="cuda", generator=g) * 2 - 1
    C0 = torch.rand((M, N), device="cuda", generator=g) * 2 - 1
    ref = 0.5 * C0.double() - 1.0 * (A.double() @ B.double().T)
    for mode in ("blocked", "tf32x6"):
        C = lib.gemm_nt_device(A, B, mode=mode, C=C0.clone(), alpha=-1.0, beta=0.5)
        assert float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref)) <= 2e-5


@pytest.mark.parametrize("mode", ["tf32x6", "tf32x3"])
def test_gemm_narrow_output(lib, cuda, mode):
    """N <= 32 (32-wide tensor-core tiles), long K (split-K partials)."""
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(3)
    M, N, K = 520, 24, 1536
    A = torch.rand((M, K), device="cuda", generator=g) * 2 - 1
    B = torch.rand((N, K), device="cuda", generator=g) * 2 - 1
    ref = A.double() @ B.double().T
    C = lib.gemm_nt_device(A, B, mode=mode)
    assert float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref)) <= 5e-6


@pytest.mark.parametrize("mode", ["tf32x6", "tf32x3"])
@pytest.mark.parametrize("M,N,K,beta", [(3000, 1700, 96, 0.0), (3000, 1700, 96, 1.0), (2900, 64, 2048, 0.0),
                                        (1500, 300, 200, 0.5), (20000, 24, 96, 0.0), (20000, 24, 96, 1.0)])
def test_gemm_persistent_tiles(lib, cuda, mode, M, N, K, beta):
    """More tiles (or K slices) than SMs, so every persistent CTA runs several
    in a row: the stage ring and the accumulator pair carry on across tiles, and
    the chunked TMA epilogue (beta 0 store, beta 1 reduce-add), the split-K
    partials (narrow N, long K), the per-thread update (other beta) and the
    32-wide tiles (N = 24: 157 tiles of 128 x 32) all see a CTA's second and
    later tiles.  Ragged M, N, K."""
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.rand((M, K), device="cuda", generator=g) * 2 - 1
    B = torch.rand((N, K), device="cuda", generator=g) * 2 - 1
    C0 = torch.rand((M, N), device="cuda", generator=g) * 2 - 1
    ref = beta * C0.double() - (A.double() @ B.double().T)
    C = lib.gemm_nt_device(A, B, mode=mode, C=C0.clone(), alpha=-1.0, beta=beta)
    torch.cuda.synchronize()
    err = float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref))
    assert err <= (3e-6 if mode == "tf32x6" else 6e-6), err
