"""Runs SVDs of one seeded matrix through the device API, for profilers.

    python -m ddcsvd.profile --size 4096 --mode tf32x6 --reps 2 [--kind graded|uniform]
    python -m ddcsvd.profile --batched 2048 --reps 2

--batched runs the seeded uneven batch instead (rng(3): m ~ U{16..256},
n ~ U{8..m}, entries U[-1, 1]) through ddcsvd_svd_batched_f32_device.

The first repetition warms up (workspace allocation, module load); each
repetition is one complete SVD.  Prints the per-SVD device time of the last
repetition.  Used by the ncu captures summarised under profiles/.
"""
from __future__ import annotations

import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main() -> None:
    import torch

    import ddcsvd

    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--cols", type=int, default=0, help="n (default: square)")
    ap.add_argument("--mode", default="tf32x6")
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--kind", default="graded", choices=["graded", "uniform"])
    ap.add_argument("--batched", type=int, default=0, help="number of problems of the uneven batch")
    args = ap.parse_args()
    if args.batched:
        import numpy as np

        torch.cuda.set_device(0)
        rng = np.random.default_rng(3)
        mats = []
        for _ in range(args.batched):
            m = int(rng.integers(16, 257))
            n = int(rng.integers(8, m + 1))
            mats.append(rng.uniform(-1, 1, (m, n)).astype(np.float32))
        plan = ddcsvd.BatchPlan([a.shape for a in mats])
        plan.load([torch.from_numpy(a).cuda() for a in mats])
        ms = 0.0
        for _ in range(args.reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            plan.run()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
        print(f"batched {args.batched}: {ms:.3f} ms")
        return
    m = args.size
    n = args.cols or m
    import numpy as np

    torch.cuda.set_device(0)
    rng = np.random.default_rng(1)
    if args.kind == "graded":  # host LAPACK: the matrix is built before any library kernel runs
        Q1, _ = np.linalg.qr(rng.standard_normal((m, n)))
        Q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
        s = 10.0 ** (-6.0 * np.arange(n) / max(n - 1, 1))
        A = torch.from_numpy(((Q1 * s) @ Q2.T).astype(np.float32)).cuda()
    else:
        A = torch.from_numpy(rng.uniform(-1, 1, (m, n)).astype(np.float32)).cuda()
    h = ddcsvd.Handle()
    Ac = A.t().contiguous()
    k = min(m, n)
    bufs = (torch.empty(k, device="cuda"), torch.empty((k, m), device="cuda"), torch.empty((k, n), device="cuda"))
    ms = 0.0
    for _ in range(args.reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ddcsvd.svd_device_colmajor(h, m, n, Ac, *bufs, mode=args.mode)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
    print(f"svd {m}x{n} mode={args.mode}: {ms:.3f} ms")


if __name__ == "__main__":
    main()
