"""The BLAS builder's sort (sft__sort_build_items, sofren2.c:2895-2924: quicksort, middle element
as pivot, Hoare scans) restated in the rank form the device kernels compute, checked against the
sequential algorithm on the CPU.

Rank form of one partition of keys a[0..n) with pivot p = a[n // 2]: the left scan stops at the
positions with fi = !(a < p) in increasing order (Lpos), the right scan at the positions with
fj = !(a > p) in decreasing order (Rpos); the k-th stops swap while Lpos[k] <= Rpos[k] (K pairs,
K >= 1 since the pivot stops both scans); afterwards i = Lpos[K-1] + 1, j = Rpos[K-1] - 1, and if
i <= j the scans stop once more without a swap, at i = min(Lpos[K], Rpos[K-1]) and
j = max(Rpos[K], Lpos[K-1]).  The parts [0, j] and [i, n) recurse."""
import numpy as np
import pytest


def sequential_sort(keys: np.ndarray, ids: np.ndarray, lo: int, n: int) -> None:
    """The reference's quicksort, recursion as an explicit stack (the order of the two recursive
    calls does not matter: their ranges are disjoint)."""
    stack = [(lo, n)]
    while stack:
        b, c = stack.pop()
        if c <= 1:
            continue
        p = keys[b + c // 2]
        i, j = 0, c - 1
        while i <= j:
            while keys[b + i] < p:
                i += 1
            while keys[b + j] > p:
                j -= 1
            if i <= j:
                keys[[b + i, b + j]] = keys[[b + j, b + i]]
                ids[[b + i, b + j]] = ids[[b + j, b + i]]
                i += 1
                j -= 1
        if j > 0:
            stack.append((b, j + 1))
        if i < c:
            stack.append((b + i, c - i))


def rank_partition(keys: np.ndarray, ids: np.ndarray, b: int, c: int) -> tuple[int, int]:
    """One partition in rank form, vectorised: returns the scans' final (i, j), relative to b."""
    seg = keys[b:b + c]
    p = seg[c // 2]
    fi = ~(seg < p)
    fj = ~(seg > p)
    lpos = np.flatnonzero(fi)                  # left stops in order
    rpos = np.flatnonzero(fj)[::-1]            # right stops from the end
    m = min(len(lpos), len(rpos))
    K = int(np.count_nonzero(lpos[:m] <= rpos[:m]))   # a prefix: lpos rises, rpos falls
    assert K >= 1
    a, z = b + lpos[:K], b + rpos[:K]
    keys[a], keys[z] = keys[z].copy(), keys[a].copy()
    ids[a], ids[z] = ids[z].copy(), ids[a].copy()
    i, j = int(lpos[K - 1]) + 1, int(rpos[K - 1]) - 1
    if i <= j:
        l_next = int(lpos[K]) if K < len(lpos) else 1 << 30
        r_next = int(rpos[K]) if K < len(rpos) else -1
        i = min(l_next, int(rpos[K - 1]))
        j = max(r_next, int(lpos[K - 1]))
    return i, j


def rank_sort(keys: np.ndarray, ids: np.ndarray) -> None:
    """Rounds over disjoint pieces, as the device does them."""
    pieces = [(0, len(keys))] if len(keys) > 1 else []
    while pieces:
        nxt = []
        for b, c in pieces:
            i, j = rank_partition(keys, ids, b, c)
            if j >= 1:
                nxt.append((b, j + 1))
            if c - i >= 2:
                nxt.append((b + i, c - i))
        pieces = nxt


def _keys(kind: str, n: int, rng) -> np.ndarray:
    if kind == "ties":
        return rng.integers(0, 4, n).astype(np.float32)
    if kind == "spread":
        return (rng.integers(0, 100000, n) * np.float32(0.01)).astype(np.float32)
    if kind == "sorted":
        return np.arange(n, dtype=np.float32)
    if kind == "reversed":
        return np.arange(n, 0, -1).astype(np.float32)
    if kind == "nan":
        k = rng.integers(0, 8, n).astype(np.float32)
        k[rng.random(n) < 0.1] = np.nan
        return k
    if kind == "zeros":
        return np.where(rng.random(n) < 0.5, np.float32(0.0), np.float32(-0.0)).astype(np.float32)
    if kind == "equal":
        return np.full(n, 1.5, np.float32)
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["ties", "spread", "sorted", "reversed", "nan", "zeros", "equal"])
def test_rank_form_equals_sequential_quicksort(kind):
    rng = np.random.default_rng(2895 + sum(map(ord, kind)))
    for n in list(range(1, 40)) + [64, 127, 128, 129, 1000, 3001]:
        k0 = _keys(kind, n, rng)
        ka, ia = k0.copy(), np.arange(n)
        kb, ib = k0.copy(), np.arange(n)
        sequential_sort(ka, ia, 0, n)
        rank_sort(kb, ib)
        assert np.array_equal(ia, ib), f"{kind} n={n}: the permutations differ"
