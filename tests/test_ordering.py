"""The incremental ordering's position formulas (aep_sort.cu), restated in numpy:
for random ascending previous keys with a random set of changed keys, stayers at
(stayers before them) + (movers with a smaller key) and movers at (their (key,
slot) rank) + (stayers with key <= theirs) form a permutation that sorts the new
keys, with the mover list in any order.  The GPU kernels are checked against the
full radix sort in tests/test_parity_gpu.py."""
import numpy as np


def incremental_order(prev, keys, rng, block=1024):
    n = len(keys)
    mover = keys != prev
    movers = np.nonzero(mover)[0]
    order = rng.permutation(len(movers))  # the list is appended by atomics: any order
    mk, mj = keys[movers][order], movers[order]
    nb = (n + block - 1) // block
    blk = np.array([mover[b * block:(b + 1) * block].sum() for b in range(nb)], np.int64)
    blk_off = np.concatenate([[0], np.cumsum(blk)[:-1]])
    out_k = np.full(n, -1, np.int64)
    out_p = np.full(n, -1, np.int64)
    mkeys_sorted = np.zeros(len(movers), np.int64)
    for ki, ji in zip(mk, mj):
        rank = np.sum((mk < ki) | ((mk == ki) & (mj < ji)))
        pos = rank + np.searchsorted(prev, ki, side="right") - np.sum(prev[mj] <= ki)
        mkeys_sorted[rank] = ki
        out_k[pos], out_p[pos] = ki, ji
    for j in np.nonzero(~mover)[0]:
        b = j // block
        before = blk_off[b] + mover[b * block:j].sum()
        pos = j - before + np.searchsorted(mkeys_sorted, keys[j], side="left")
        assert out_p[pos] == -1
        out_k[pos], out_p[pos] = keys[j], j
    return out_k, out_p


def test_incremental_order_is_a_sorting_permutation():
    rng = np.random.default_rng(0)
    for _ in range(60):
        n = int(rng.integers(1, 3000))
        prev = np.sort(rng.integers(0, 200, n))
        keys = prev.copy()
        idx = rng.choice(n, size=int(rng.integers(0, max(1, n // 4))), replace=False)
        keys[idx] = rng.integers(0, 200, len(idx))
        ok, op = incremental_order(prev, keys, rng)
        assert sorted(op) == list(range(n))
        assert np.all(np.diff(ok) >= 0) and np.array_equal(ok, keys[op])
        # stayers keep slot order among equal keys and come before movers
        for k in np.unique(ok):
            slots = op[ok == k]
            stay = slots[keys[slots] == prev[slots]]
            assert np.all(np.diff(stay) > 0)
            assert np.all(keys[slots[:len(stay)]] == prev[slots[:len(stay)]])
