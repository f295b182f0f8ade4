"""CPU check of the error bound that lets the D&C pick a secular root's origin
pole from FP32 sums (ddc-svd_gb300/csrc/dc.cu, sec_mid32): whenever |f32| at
the midpoint of (d_i, d_i+1) clears twice the bound, its sign must equal the
FP64 sign, over poles that are uniform, graded, clustered to 1e-9 and 1e-12,
tiny and huge.  The FP32 arithmetic is restated with numpy float32 (IEEE
round-to-nearest; the GPU may contract the product and the subtraction into
one FMA, which only removes a rounding the bound allows for)."""
import numpy as np
import pytest

E32 = np.float32(np.finfo(np.float32).eps)


def mid32(d, z, i):
    """f at the midpoint and its bound, as sec_mid32 computes them."""
    q = len(d)
    df = d.astype(np.float32)
    zf = z.astype(np.float32)
    dd = (d[i + 1] - d[i]) * (d[i + 1] + d[i])
    tau = np.float32(0.5 * dd)
    do = df[i]
    with np.errstate(all="ignore"):
        dl = (df - do) * (df + do) - tau
        tt = zf * zf / dl
        ad = np.abs(df) + np.abs(do)
        ed = np.float32(3.0) * E32 * (ad * ad + np.abs(tau))
        ok = (ed < np.float32(0.5) * np.abs(dl)) & (np.abs(dl) >= np.float32(2.0 ** -100))
        at = np.abs(tt)
        ea = np.where(ok, at * (np.float32(2.0) * ed / np.abs(dl) + np.float32(4.0) * E32), np.float32(np.inf))
        s = np.float32(0.0)
        sa = np.float32(0.0)
        e = np.float32(0.0)
        for j in range(q):  # sequential FP32 sums (the GPU's order differs; the bound holds for any order)
            s = np.float32(s + tt[j])
            sa = np.float32(sa + at[j])
            e = np.float32(e + ea[j])
        f = np.float32(1.0) + s
        err = e + np.float32(q + 2) * E32 * (np.float32(1.0) + sa)
    return f, err


def mid64(d, z, i):
    dd = (d[i + 1] - d[i]) * (d[i + 1] + d[i])
    return 1.0 + np.sum(z * z / ((d - d[i]) * (d + d[i]) - 0.5 * dd))


def poles(rng, kind, n):
    if kind == "uniform":
        d = np.sort(rng.uniform(0.01, 2.0, n))
    elif kind == "graded":
        d = np.sort(10.0 ** rng.uniform(-12, 0, n))
    elif kind in ("cluster9", "cluster12"):
        gap = 1e-9 if kind == "cluster9" else 1e-12
        base = np.sort(rng.uniform(0.5, 1.5, max(2, n // 3)))
        d = np.sort(np.concatenate([base, base * (1 + gap), base * (1 + 2 * gap)]))[:n]
    elif kind == "tiny":
        d = np.sort(rng.uniform(1e-22, 1e-18, n))
    else:  # huge
        d = np.sort(rng.uniform(1e17, 1e19, n))
    d = np.unique(d)
    return d


@pytest.mark.parametrize("kind", ["uniform", "graded", "cluster9", "cluster12", "tiny", "huge"])
def test_fp32_origin_sign_matches_fp64_when_bound_clears(kind):
    rng = np.random.default_rng(len(kind))
    used = total = 0
    for trial in range(12):
        n = int(rng.integers(3, 120))
        d = poles(rng, kind, n)
        if len(d) < 3:
            continue
        scale = np.abs(d).max()
        z = rng.standard_normal(len(d)) * scale * 10.0 ** rng.uniform(-3, 0, len(d))
        z[rng.random(len(d)) < 0.1] *= 1e-6  # some nearly deflated components
        for i in range(len(d) - 1):
            f32, err = mid32(d, z, i)
            total += 1
            if np.isfinite(f32) and abs(f32) > 2 * err:
                used += 1
                f64 = mid64(d, z, i)
                assert (f32 >= 0) == (f64 >= 0), (kind, trial, i, float(f32), float(err), f64)
    assert total > 0
    if kind in ("uniform", "graded"):
        assert used > 0.5 * total  # the FP32 choice is the common case on ordinary spectra
