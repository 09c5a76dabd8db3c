"""The index arithmetic of the coherent sort (csrc/coherent_sort.cu), restated
in numpy and checked against a stable argsort on CPU: for keys k[0..n) and any
non-decreasing hint h, "stayers" (k[i] == h[i]) land at
i - movers_before(i) + movers_below(h[i], i), and the radix-sorted "movers" at
rank + stayers_below(k, index); together they must form the stable sort of
(key, index).  Also the kernels' two searches: the 32-lane search of the
placement kernel (one pivot per lane, ballot of a prefix) and the cell-table
shortcut for a mover's insertion point, accepted only where the hint confirms
the run.  The GPU kernels themselves are checked in test_gpu_sort.py and
test_gpu_single_scale.py."""
import numpy as np
import pytest


def lane_search(pred, m):
    """32-way search of coherent_merge_kernel: count of q in [0, m) with pred(q),
    pred true on a prefix."""
    lo, hi = 0, m
    while hi - lo > 32:
        step = (hi - lo + 31) // 32
        b = [lo + l * step < hi and pred(lo + l * step) for l in range(32)]
        nb = sum(b)
        assert all(b[:nb])  # the ballot is a prefix of the lanes
        if nb == 0:
            hi = lo
        else:
            lo, hi = lo + (nb - 1) * step + 1, min(hi, lo + nb * step)
    return lo + sum(1 for l in range(32) if lo + l < hi and pred(lo + l))


def insertion_point(hint, k, v, cell_run=None):
    """First q with (hint[q], q) >= (k, v); cell_run = a claimed (start, end) of
    key k, used only where the hint confirms it (a stale table is harmless)."""
    n = hint.size
    if cell_run is not None:
        s, e = cell_run
        if s < e <= n and hint[s] == k and hint[e - 1] == k and (s == 0 or hint[s - 1] < k) \
                and (e == n or hint[e] > k):
            return min(max(v, s), e)
    lo, hi = 0, n
    while lo < hi:
        mid = (lo + hi) // 2
        if hint[mid] < k or (hint[mid] == k and mid < v):
            lo = mid + 1
        else:
            hi = mid
    return lo


def coherent_sort(keys, hint, cell_table=None):
    n = keys.size
    mover = keys != hint
    before = np.concatenate([[0], np.cumsum(mover)])  # movers with index < q
    mi = np.nonzero(mover)[0]
    order = np.argsort(keys[mi], kind="stable")
    smk, smv = keys[mi][order], mi[order]
    m = mi.size
    out_k = np.full(n, -1, np.int64)
    out_v = np.full(n, -1, np.int64)
    for i in np.nonzero(~mover)[0]:
        key = hint[i]
        below = lane_search(lambda q: smk[q] < key or (smk[q] == key and smv[q] < i), m)
        d = i - before[i] + below
        assert out_k[d] == -1
        out_k[d], out_v[d] = key, i
    for r in range(m):
        k, v = smk[r], smv[r]
        run = cell_table(k) if cell_table else None
        q = insertion_point(hint, k, v, run)
        d = r + q - before[q]
        assert out_k[d] == -1
        out_k[d], out_v[d] = k, v
    return out_k, out_v


@pytest.mark.parametrize("case", range(8))
def test_coherent_placement_is_the_stable_sort_for_any_hint(case):
    rng = np.random.default_rng(case)
    n = int(rng.integers(1, 700))
    nk = int(rng.integers(1, 60))
    hint = np.sort(rng.integers(0, nk, n))
    if case % 4 == 0:
        keys = rng.integers(0, nk, n)  # unrelated to the hint
    elif case % 4 == 1:
        keys = hint.copy()  # nothing changed
    elif case % 4 == 2:
        keys = hint.copy()
        idx = rng.choice(n, max(1, n // 25), replace=False)
        keys[idx] = rng.integers(0, nk, idx.size)  # a few changed
    else:
        hint = np.full(n, 2**32 - 1)  # creation: every key changed
        keys = rng.integers(0, nk, n)
    ok, ov = coherent_sort(keys, hint)
    ref = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(ov, ref)
    np.testing.assert_array_equal(ok, keys[ref])


def test_lane_search_counts_the_true_prefix():
    rng = np.random.default_rng(5)
    for m in (0, 1, 31, 32, 33, 1023, 1024, 1025, 7000, 12289, 40000):
        for ans in {0, m, int(rng.integers(0, m + 1))}:
            assert lane_search(lambda q: q < ans, m) == ans


def test_stale_or_garbage_cell_table_gives_the_same_result():
    rng = np.random.default_rng(9)
    n, nk = 500, 40
    hint = np.sort(rng.integers(0, nk, n))
    keys = hint.copy()
    idx = rng.choice(n, 40, replace=False)
    keys[idx] = rng.integers(0, nk, idx.size)
    true_runs = {k: (int(np.searchsorted(hint, k, "left")), int(np.searchsorted(hint, k, "right")))
                 for k in range(nk)}
    ref = np.argsort(keys, kind="stable")
    tables = {
        "exact": lambda k: true_runs[k] if true_runs[k][0] < true_runs[k][1] else (2**32 - 1, 2**32 - 1),
        "stale": lambda k: (true_runs[k][0] + 1, true_runs[k][1]),
        "garbage": lambda k: tuple(int(x) for x in rng.integers(0, n + 3, 2)),
    }
    for name, table in tables.items():
        _, ov = coherent_sort(keys, hint, table)
        np.testing.assert_array_equal(ov, ref, err_msg=name)
