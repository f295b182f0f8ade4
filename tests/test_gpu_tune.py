"""Launch-configuration autotuner: knob access, the two tuners, and that a
tuned handle still produces parity-level results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _check(orc, A, s, U, V):
    A64 = np.asarray(A, dtype=np.float64)
    met = orc.metrics(A64, s, U, V, np.linalg.svd(A64, compute_uv=False))
    assert met["sig_abs"] <= TOL and met["resid"] <= TOL and met["orth_u"] <= TOL and met["orth_v"] <= TOL, met


def test_tuning_roundtrip(lib, cuda):
    h = lib.Handle()
    t0 = h.tuning
    assert t0 == {"splitk_max": 16, "tc_bn": 0, "batch_threads": 512, "batch_smem_full": 1, "dc_terms": 8,
                  "tall_qr": 2, "panel_fused": 1, "panel_tail": 512}
    h.tuning = {"splitk_max": 4, "dc_terms": 16}
    assert h.tuning["splitk_max"] == 4 and h.tuning["dc_terms"] == 16 and h.tuning["tc_bn"] == 0
    h.tuning = t0
    assert h.tuning == t0


def test_autotune_svd_then_parity(lib, cuda, orc):
    torch = cuda
    h = lib.Handle()
    t = h.autotune_svd(640, 384, mode="tf32x6", reps=1)
    assert t["splitk_max"] in (1, 2, 4, 8, 16) and t["tc_bn"] in (0, 64)
    rng = np.random.default_rng(5)
    A = rng.uniform(-1, 1, (640, 384)).astype(np.float32)
    k = 384
    Ac = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    bufs = (torch.empty(k, device="cuda"), torch.empty((k, 640), device="cuda"), torch.empty((k, 384), device="cuda"))
    lib.svd_device_colmajor(h, 640, 384, Ac, *bufs, mode="tf32x6")
    torch.cuda.synchronize()
    s, Ut, Vt = (x.double().cpu().numpy() for x in bufs)
    _check(orc, A, s, Ut.T, Vt.T)


def test_autotune_batched_then_parity(lib, cuda, orc):
    torch = cuda
    rng = np.random.default_rng(9)
    shapes = []
    mats = []
    for _ in range(48):
        m = int(rng.integers(16, 129))
        n = int(rng.integers(8, m + 1))
        shapes.append((m, n))
        mats.append(rng.uniform(-1, 1, (m, n)).astype(np.float32))
    h = lib.Handle()
    t = h.autotune_batched(shapes, reps=1)
    assert t["batch_threads"] in (256, 512) and t["batch_smem_full"] in (0, 1) and t["dc_terms"] in (4, 8, 16)
    plan = lib.BatchPlan(shapes, handle=h)
    plan.load([torch.from_numpy(a).cuda() for a in mats])
    plan.run()
    torch.cuda.synchronize()
    for b in range(0, len(mats), 5):
        s, U, V = (x.double().cpu().numpy() for x in plan.result(b))
        _check(orc, mats[b], s, U, V)
