"""CPU tests of the library's host-side planning of stage 2 (no GPU work):
the splitting of the bidiagonal and the D&C forest with its schedule, through
ddcsvd_split_plan / ddcsvd_dc_plan, against a restatement of the reference's
recursion (Calculations-Parallel.c:706-850: an N x (N+1) node splits at
K = N/2 into a K x (K+1) and an (N-K-1) x (N-K) child, rows [r, r+K) and
[r+K+1, r+N); leaves have N <= 2) and the schedule's own invariants."""
import numpy as np
import pytest

EPS64 = float(np.finfo(np.float64).eps)
EPS32 = float(np.finfo(np.float32).eps)


def _a(x):
    return x.ctypes.data


def split_plan(L, a, b, eps):
    a = np.array(a, dtype=np.float64)
    b = np.array(b, dtype=np.float64)
    N = len(a)
    starts = np.zeros(N + 1, dtype=np.int32)
    ns = np.zeros(1, dtype=np.int32)
    assert L.ddcsvd_split_plan(N, _a(a), _a(b), eps, _a(starts), _a(ns)) == 0
    return a, b, starts[: ns[0]].tolist()


def dc_plan(L, N, starts, tpl=8):
    st = np.asarray(starts, dtype=np.int32)
    meta = np.zeros(8, dtype=np.int32)
    assert L.ddcsvd_dc_plan(N, len(st), _a(st), tpl, None, 0, _a(meta)) == 1  # cap 0: too small, meta filled
    out = np.zeros(int(meta[7]), dtype=np.int32)
    assert L.ddcsvd_dc_plan(N, len(st), _a(st), tpl, _a(out), len(out), _a(meta)) == 0
    nnodes, md, ndm, ntrees, nseg, maxtree, toff, total = (int(x) for x in meta)
    o = 0

    def take(k):
        nonlocal o
        v = out[o:o + k]
        o += k
        return v

    T = {}
    for name in ("r0", "nn", "slot", "K", "c1", "c2"):
        T[name] = take(nnodes)
    T["ds"], T["dms"] = take(md + 2), take(md + 2)
    T["dmerge"], T["dgroup"] = take(ndm), take(md + 2)
    assert o == toff
    T["tree_seg"], T["seg_lo"] = take(ntrees + 1), take(nseg + 1)
    T["seg_mid"], T["seg_depth"], T["seg_G"] = take(nseg), take(nseg), take(nseg)
    T["nodes_out"], T["order"] = take(nnodes), take(ntrees)
    assert o == total
    T.update(nnodes=nnodes, md=md, ntrees=ntrees, nseg=nseg, maxtree=maxtree, tpl=tpl)
    return T


def ref_nodes(lo, n, d, out):
    """The reference's recursion: (first row, size, depth, K or -1)."""
    k = n // 2 if n > 2 else -1
    out.append((lo, n, d, k))
    if n > 2:
        ref_nodes(lo, k, d + 1, out)
        ref_nodes(lo + k + 1, n - k - 1, d + 1, out)


def lanes(mx, tpl):
    G = 1
    while G < 32 and G * tpl < mx:
        G <<= 1
    return G


def check_plan(T, N, starts):
    n = T["nnodes"]
    depth = np.zeros(n, dtype=int)
    for d in range(T["md"] + 1):
        depth[T["ds"][d]:T["ds"][d + 1]] = d
    assert T["ds"][0] == 0 and T["ds"][T["md"] + 1] == n
    # the nodes are the reference's recursion over the blocks
    want = []
    blocks = [(lo, hi) for lo, hi in zip(starts[:-1], starts[1:]) if hi > lo]
    for lo, hi in blocks:
        ref_nodes(lo, hi - lo, 0, want)
    got = sorted(zip(T["r0"].tolist(), T["nn"].tolist(), depth.tolist(), T["K"].tolist()))
    assert got == sorted(want)
    for d in range(T["md"] + 1):  # slots ascending within a depth
        sl = T["slot"][T["ds"][d]:T["ds"][d + 1]]
        assert np.all(np.diff(sl) > 0)
    # children: (r0, K) and (r0 + K + 1, n - K - 1), one depth down; leaves have none
    for i in range(n):
        k = T["K"][i]
        if k < 0:
            assert T["nn"][i] <= 2 and T["c1"][i] == -1 and T["c2"][i] == -1
            continue
        a, b = T["c1"][i], T["c2"][i]
        assert (T["r0"][a], T["nn"][a], depth[a]) == (T["r0"][i], k, depth[i] + 1)
        assert (T["r0"][b], T["nn"][b], depth[b]) == (T["r0"][i] + k + 1, T["nn"][i] - k - 1, depth[i] + 1)
    # merge lists and lanes per root by depth
    for d in range(T["md"] + 1):
        m = T["dmerge"][T["dms"][d]:T["dms"][d + 1]].tolist()
        assert m == [i for i in range(T["ds"][d], T["ds"][d + 1]) if T["K"][i] >= 0]
        mx = max([T["nn"][i] for i in m], default=0)
        assert T["dgroup"][d] == lanes(mx, T["tpl"])
    # per-tree schedule: every node once, in its block; deepest segment first,
    # merges before leaves in a segment; trees by size, largest first
    assert T["ntrees"] == len(blocks)
    assert sorted(T["nodes_out"].tolist()) == list(range(n))
    sizes = []
    for t, (lo, hi) in enumerate(blocks):
        s0, s1 = T["tree_seg"][t], T["tree_seg"][t + 1]
        prev = None
        for s in range(s0, s1):
            seg = T["nodes_out"][T["seg_lo"][s]:T["seg_lo"][s + 1]]
            mid = T["seg_mid"][s] - T["seg_lo"][s]
            assert all(T["K"][i] >= 0 for i in seg[:mid]) and all(T["K"][i] < 0 for i in seg[mid:])
            assert all(depth[i] == T["seg_depth"][s] for i in seg)
            assert all(lo <= T["r0"][i] and T["r0"][i] + T["nn"][i] <= hi for i in seg)
            assert T["seg_G"][s] == lanes(max([T["nn"][i] for i in seg[:mid]], default=0), T["tpl"])
            if prev is not None:
                assert T["seg_depth"][s] < prev
            prev = T["seg_depth"][s]
        assert prev == 0  # the root's segment is last
        sizes.append(hi - lo)
    order = T["order"].tolist()
    assert sorted(order) == list(range(len(blocks)))
    assert [sizes[t] for t in order] == sorted(sizes, key=lambda x: -x)
    assert order == sorted(range(len(blocks)), key=lambda t: -sizes[t])  # stable
    assert T["maxtree"] == max(sizes)


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 17, 64, 257, 1000, 4096])
def test_dc_plan_single_block_is_the_reference_recursion(lib, N):
    L = lib.load()
    check_plan(dc_plan(L, N, [0, N]), N, [0, N])


@pytest.mark.parametrize("tpl", [4, 8, 16])
def test_dc_plan_batch_forest(lib, tpl):
    """Many blocks of uneven sizes (singletons and pairs included), as a
    batch of problems or a split bidiagonal gives."""
    rng = np.random.default_rng(tpl)
    sizes = [1, 2, 3] + rng.integers(1, 300, 200).tolist()
    starts = np.concatenate([[0], np.cumsum(sizes)]).tolist()
    L = lib.load()
    check_plan(dc_plan(L, starts[-1], starts, tpl), starts[-1], starts)


def test_dc_plan_rejects_bad_starts(lib):
    L = lib.load()
    meta = np.zeros(8, dtype=np.int32)
    for st in ([1, 10], [0, 9], [0, 6, 4, 10]):
        s = np.asarray(st, dtype=np.int32)
        assert L.ddcsvd_dc_plan(10, len(s), _a(s), 8, None, 0, _a(meta)) == 1


def test_split_plan_thresholds(lib):
    """Splits at |b_i| <= 4 eps max|entry| (the pipeline's rule), zeroes those
    entries and the last one, and leaves the rest alone."""
    L = lib.load()
    rng = np.random.default_rng(2)
    N = 50
    a = rng.uniform(0.5, 1.5, N)
    b = rng.uniform(0.5, 1.5, N)
    b[5], b[20], b[30], b[40] = 0.0, 1e-20, 3e-16, 1e-14
    mx = max(np.abs(a).max(), np.abs(b[:-1]).max())
    a64, b64, st = split_plan(L, a, b, EPS64)
    cut = [i for i in range(N - 1) if abs(b[i]) <= 4 * EPS64 * mx]
    assert cut == [5, 20, 30]
    assert st == [0] + [i + 1 for i in cut] + [N]
    assert np.all(b64[cut] == 0.0) and b64[N - 1] == 0.0 and b64[40] == 1e-14
    assert np.array_equal(a64, a)
    _, b32, st32 = split_plan(L, a, b, EPS32)  # the FP32 pipeline's tolerance also cuts 1e-14
    assert st32 == [0, 6, 21, 31, 41, N] and b32[40] == 0.0


def test_split_plan_feeds_dc_plan(lib):
    """A split bidiagonal's blocks become the trees of the forest."""
    L = lib.load()
    rng = np.random.default_rng(4)
    N = 300
    a = rng.uniform(0.5, 1.5, N)
    b = rng.uniform(0.5, 1.5, N)
    b[rng.choice(N - 1, 25, replace=False)] = 0.0
    _, _, st = split_plan(L, a, b, EPS32)
    check_plan(dc_plan(L, N, st), N, st)


@pytest.mark.parametrize("eps", [EPS64, EPS32])
def test_split_plan_matches_oracle(lib, orc, eps):
    """The library's host split and the oracle's (oracle/ddcsvd_oracle.c,
    orc_bdsvd) zero exactly the same superdiagonal entries."""
    L = lib.load()
    rng = np.random.default_rng(int(eps * 1e20) % 1000)
    for trial in range(20):
        N = int(rng.integers(2, 400))
        a = rng.uniform(-2, 2, N) * 10.0 ** rng.uniform(-8, 0, N)
        b = rng.uniform(-2, 2, N) * 10.0 ** rng.uniform(-20, 0, N)
        _, b_lib, _ = split_plan(L, a, b, eps)
        _, _, b_orc = orc.bdsvd(a, b[: N - 1], eps)
        assert np.array_equal(b_lib[: N - 1] == 0.0, b_orc == 0.0), trial
