"""Seeded random shapes through every tensor-core path at once (GPU).

Each draw picks m, n in [1, 1500] (tall, wide and square alike), a value
distribution, a mode and whether the QR-first path is forced, so that the
256-reflector back-transformation blocks meet full, partial and single
128-blocks, the side stream's preparation and the host-buffer copies run
on uneven layouts, and the wide path swaps its factors.  Every result must
meet the FP64 bounds of the single-matrix tests."""
import numpy as np
import pytest

from test_gpu_svd import _mode_available, check_metrics

pytestmark = pytest.mark.gpu


def _draw(seed):
    rng = np.random.default_rng(1000 + seed)
    m, n = (int(x) for x in rng.integers(1, 1501, 2))
    kind = ["uniform", "normal", "lowrank"][seed % 3]
    if kind == "uniform":
        A = rng.uniform(-1, 1, (m, n))
    elif kind == "normal":
        A = rng.standard_normal((m, n)) * 10.0 ** rng.integers(-3, 4)
    else:
        r = int(rng.integers(1, min(m, n) + 1))
        A = rng.uniform(-1, 1, (m, r)) @ rng.uniform(-1, 1, (r, n))
    return A.astype(np.float32), ["tf32x3", "tf32x6"][seed % 2], int(rng.integers(0, 2))


@pytest.mark.parametrize("seed", range(24))
def test_random_shape_device_api(lib, cuda, orc, seed):
    A, mode, tall_qr = _draw(seed)
    if not _mode_available(lib, mode):
        pytest.skip(f"{mode} unavailable")
    h = lib.Handle()
    h.tuning = {"tall_qr": tall_qr}
    s, U, V = lib.svd_device(cuda.from_numpy(A).cuda(), mode=mode, handle=h)
    cuda.cuda.synchronize()
    check_metrics(orc, A, s.double().cpu().numpy(), U.double().cpu().numpy(), V.double().cpu().numpy())


@pytest.mark.parametrize("seed", range(24, 32))
def test_random_shape_host_api(lib, cuda, orc, seed):
    """The host-buffer FP32 entry point (its early copy of V, or of U for a
    wide input, runs on the side stream)."""
    A, mode, _ = _draw(seed)
    if not _mode_available(lib, mode):
        pytest.skip(f"{mode} unavailable")
    s, U, V = lib.svd(A, mode=mode)
    check_metrics(orc, A, s.astype(np.float64), U.astype(np.float64), V.astype(np.float64))
