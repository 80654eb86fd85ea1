"""The dense path's flat work lists, checked on the CPU.

k_dense_refine_scan writes exclusive offsets of per-query item counts
(sparsedist_gb300/csrc/sdg_dense.cu): for the FP32 cut, ceil(count / 8) items
for each query with more than k candidates; for the exact values, one item
per candidate of every query.  k_dense_refine_dot and k_dense_values_flat
find an item's query by a binary search for the last offset <= the item, and
persistent warps take items w, w + W, w + 2W, ...  Restated here in numpy:
every candidate slot that needs work is visited exactly once, no other slot
is, and every slot index stays inside its query's [0, count) range.
"""
import numpy as np

RG = 8


def scan(counts, k, unit):
    if unit == 1:
        items = counts.astype(np.int64)
    else:
        items = np.where(counts > k, (counts + unit - 1) // unit, 0).astype(np.int64)
    off = np.zeros(len(counts) + 1, np.int64)
    off[1:] = np.cumsum(items)
    return off


def find_query(off, it):
    lo, hi = 0, len(off) - 1                      # off[lo] <= it < off[hi]
    while hi - lo > 1:
        mid = (lo + hi) >> 1
        if off[mid] <= it:
            lo = mid
        else:
            hi = mid
    return lo


def visit_cut_items(counts, k, cap, warps):
    off = scan(counts, k, RG)
    seen = np.zeros((len(counts), cap), np.int32)
    items = int(off[-1])
    for w in range(warps):
        for it in range(w, items, warps):
            ql = find_query(off, it)
            t0 = (it - off[ql]) * RG
            n = min(RG, counts[ql] - t0)
            assert counts[ql] > k and 1 <= n <= RG and t0 + n <= counts[ql] <= cap
            seen[ql, t0:t0 + n] += 1
    return seen


def visit_value_pairs(counts, cap, warps):
    off = scan(counts, 0, 1)
    seen = np.zeros((len(counts), cap), np.int32)
    total = int(off[-1])
    for w in range(warps):
        for base in range(w * 32, total, warps * 32):
            for lane in range(min(32, total - base)):
                f = base + lane
                ql = find_query(off, f)
                t = f - off[ql]
                assert 0 <= t < counts[ql] <= cap
                seen[ql, t] += 1
    return seen


def test_cut_items_cover_each_needed_slot_once():
    rng = np.random.default_rng(5)
    for k, cap, nq, warps in [(20, 1536, 300, 37), (1, 512, 50, 3), (64, 4352, 120, 64), (1024, 16384, 9, 5)]:
        counts = rng.integers(0, cap + 1, nq)
        counts[::7] = 0                            # degenerate or overflowing queries
        counts[1::11] = k                          # exactly k: no cut
        counts[2::13] = k + 1
        counts[3::17] = cap
        seen = visit_cut_items(counts, k, cap, warps)
        want = np.zeros_like(seen)
        for q, c in enumerate(counts):
            if c > k:
                want[q, :c] = 1
        assert np.array_equal(seen, want)


def test_value_pairs_cover_each_candidate_once():
    rng = np.random.default_rng(9)
    for cap, nq, warps in [(1536, 400, 29), (512, 1, 1), (512, 64, 200)]:
        counts = rng.integers(0, 60, nq)
        counts[::5] = 0
        seen = visit_value_pairs(counts, cap, warps)
        want = np.zeros_like(seen)
        for q, c in enumerate(counts):
            want[q, :c] = 1
        assert np.array_equal(seen, want)


def test_empty_work_lists():
    assert scan(np.zeros(10, np.int64), 20, RG)[-1] == 0
    assert visit_cut_items(np.full(4, 20), 20, 512, 8).sum() == 0
    assert visit_value_pairs(np.zeros(3, np.int64), 512, 4).sum() == 0
