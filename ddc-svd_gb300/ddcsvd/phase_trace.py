"""Per-phase timing of the persistent kernels from a tracing build.

    python -m ddcsvd.phase_trace --size 4096          # panel kernel, column 5 of every panel
    python -m ddcsvd.phase_trace --size 4096 --allcols  # every column of the panels at k0 = 0, 1024, ...
    python -m ddcsvd.phase_trace --batched 2048       # D&C kernel phases per depth, batched workload

Builds a second copy of the library with -DDDCSVD_PHASE_TRACE (into
ddcsvd/_lib_trace/, separate from the product library), runs two SVDs and
prints the %globaltimer intervals that one CTA recorded between its phase
marks.  The marks compile to nothing in the product build.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from ddcsvd import build as _build  # noqa: E402

PANEL = ["S1", "B1wait", "S2", "S3stage", "S3dots", "S3tail", "B2wait", "S5", "S5stage", "S6gemv", "S6tail"]
DC = ["P1", "B1", "P2", "B2", "P3", "B3", "P4", "B4", "P5", "B5"]


def build_trace(allcols: bool) -> str:
    nvcc = _build._nvcc()
    out = os.path.join(HERE, "_lib_trace", "allcols" if allcols else "default")
    os.makedirs(out, exist_ok=True)
    defs = ["-DDDCSVD_PHASE_TRACE"] + (["-DDDCSVD_TRACE_ALLCOLS"] if allcols else [])

    def comp(src):
        obj = os.path.join(out, os.path.basename(src) + ".o")
        subprocess.check_call([nvcc, *_build.ARCH, *_build.NVCC_FLAGS, *defs, "-I", _build.INCLUDE, "-c", src, "-o",
                               obj])
        return obj

    with cf.ThreadPoolExecutor(8) as ex:
        objs = list(ex.map(comp, _build.sources()))
    lib = os.path.join(out, "libddcsvd_trace.so")
    libdir = _build._cuda_lib_dir(nvcc)
    subprocess.check_call([nvcc, *_build.ARCH, "-shared", "-o", lib, *objs, "-cudart", "shared", f"-L{libdir}",
                           "-Xlinker", f"-rpath={libdir}", "-lcudart"])
    return lib


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--allcols", action="store_true")
    ap.add_argument("--batched", type=int, default=0)
    args = ap.parse_args()
    import torch

    import ddcsvd
    from ddcsvd import _lib

    lib = _lib.load(build_trace(args.allcols))
    if args.batched:
        rng = np.random.default_rng(3)
        mats = []
        for _ in range(args.batched):
            m = int(rng.integers(16, 257))
            n = int(rng.integers(8, m + 1))
            mats.append(rng.uniform(-1, 1, (m, n)).astype(np.float32))
        plan = ddcsvd.BatchPlan([a.shape for a in mats])
        plan.load([torch.from_numpy(a).cuda() for a in mats])
        for _ in range(2):
            plan.run()
        torch.cuda.synchronize()
    else:
        rng = np.random.default_rng(1)
        A = torch.from_numpy(rng.uniform(-1, 1, (args.size, args.size)).astype(np.float32)).cuda()
        for _ in range(2):
            ddcsvd.svd_device(A, mode="tf32x6")
        torch.cuda.synchronize()
    # D&C: one row per depth
    buf = (ctypes.c_ulonglong * (64 * 16))()
    lib.ddcsvd_dc_trace_read(buf)
    t = np.array(buf, dtype=np.float64).reshape(64, 16)
    print("D&C phases (us per depth, CTA 0)")
    print("  d    " + " ".join(f"{n:>7s}" for n in DC) + "    total")
    tot = np.zeros(10)
    for d in range(63, -1, -1):
        x = t[d]
        if x[0] == 0:
            continue
        seg = np.array([(x[k + 1] - x[k]) / 1e3 if (x[k] and x[k + 1]) else 0.0 for k in range(10)])
        tot += seg
        print(f"  {d:2d}   " + " ".join(f"{v:7.1f}" for v in seg) + f" {seg.sum():8.1f}")
    print("  sum  " + " ".join(f"{v:7.1f}" for v in tot) + f" {tot.sum():8.1f}")
    hist = (ctypes.c_uint * (64 * 84))()
    lib.ddcsvd_dc_iters_read(hist)
    H = np.array(hist, dtype=np.int64).reshape(64, 84)
    print("FP64 iterations per secular root (counts over both runs), by depth: mean, max, roots > 10")
    for d in range(63, -1, -1):
        row = H[d, :81]
        if row.sum() == 0:
            continue
        its = np.arange(81)
        print(f"  {d:2d}  mean {float((row * its).sum() / row.sum()):5.2f}  max {int(its[row > 0].max()):3d}  "
              f">10: {int(row[11:].sum())} of {int(row.sum())}")
    if args.batched:
        return
    buf = (ctypes.c_ulonglong * (128 * 16))()
    lib.ddcsvd_trace_read(buf)
    t = np.array(buf, dtype=np.float64).reshape(128, 16)
    print("panel kernel phases (us), CTA 7")
    print("  row   " + " ".join(f"{n:>7s}" for n in PANEL) + "   total")
    rows = []
    for r in range(128):
        x = t[r]
        if x[0] == 0 or x[11] == 0:
            continue
        d = np.diff(x[:12]) / 1e3
        rows.append(d)
        label = (f"k0={1024 * (r // 32):5d} j={r % 32:2d}" if args.allcols else f"k0={32 * r:5d}")
        if args.allcols or r % 8 == 0:
            print(f"  {label} " + " ".join(f"{v:7.2f}" for v in d) + f" {d.sum():7.2f}")
    if rows and not args.allcols:
        est = np.array(rows).sum(0) * 32 / 1e3
        print("  estimate over the factorisation (ms, x32 columns per panel):")
        print("        " + " ".join(f"{v:7.2f}" for v in est) + f" {est.sum():7.2f}")
        dur = [(t[r][13] - t[r][12]) / 1e3 for r in range(128) if t[r][12] and t[r][13]]
        print(f"  panel launches: {len(dur)}, entry->exit sum {sum(dur) / 1e3:.2f} ms")
    # cluster tail: CTA 0, every 8th tail column
    buf = (ctypes.c_ulonglong * (128 * 16))()
    if lib.ddcsvd_tail_trace_read(buf) == 0:
        t = np.array(buf, dtype=np.float64).reshape(128, 16)
        names = ["A", "bar1", "B", "bar2", "C-red", "C-x", "bar3", "D1", "bar4", "D2"]
        rows = [r for r in range(128) if t[r][0] and t[r][10]]
        if rows:
            print("cluster tail phases (us), CTA 0, every 8th column")
            print("  col   " + " ".join(f"{n:>6s}" for n in names) + "   total")
            for r in rows[::4]:
                d = np.diff(t[r][:11]) / 1e3
                print(f"  {8 * r:5d} " + " ".join(f"{v:6.2f}" for v in d) + f" {d.sum():7.2f}")


if __name__ == "__main__":
    main()
