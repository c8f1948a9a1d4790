"""The stable LSD radix sort that orders the particles (aep_sort.cu, reached through
aep_sort_pairs):

* CPU: the tile algorithm restated in numpy (per-tile digit counts, a scan per
  digit over the tiles, a scatter that ranks each tile's pairs in rounds of one
  pair per thread, by warp and lane) is a stable sort: it equals numpy's stable
  argsort;
* GPU: the kernels against numpy's stable argsort on the particle keys of the
  sand column (524,288 particles, 128^3) and of the snow + sand collision
  (2,097,152, 256^3), as the step computes them (padded base-node block << 6 |
  base node inside the block), on random keys of every width, with many equal
  keys, and at sizes around a tile (4,096 pairs).
"""
import ctypes as C

import numpy as np
import pytest

from anisotropicelastoplasticity_gb300 import capi, scenes

TILE, THREADS = 4096, 256


def tile_radix_sort(keys, key_bits):
    """numpy restatement of sort_pairs: returns the permutation (stable)."""
    n = len(keys)
    passes = (key_bits + 7) // 8
    radix = (key_bits + passes - 1) // passes
    mask = (1 << radix) - 1
    tiles = max(1, (n + TILE - 1) // TILE)
    k, v = keys.astype(np.int64).copy(), np.arange(n)
    for p in range(passes):
        d = (k >> (p * radix)) & mask
        hist = np.zeros((mask + 1, tiles), np.int64)
        for t in range(tiles):
            hist[:, t] = np.bincount(d[t * TILE:(t + 1) * TILE], minlength=mask + 1)
        totals = hist.sum(axis=1)
        row = np.cumsum(hist, axis=1) - hist  # exclusive scan of each digit's row over the tiles
        base = np.cumsum(totals) - totals
        ok, ov = np.empty_like(k), np.empty_like(v)
        for t in range(tiles):
            start = base + row[:, t]
            for r in range(TILE // THREADS):  # rounds of one pair per thread, in input order
                lo = t * TILE + r * THREADS
                for i in range(lo, min(lo + THREADS, n)):
                    ok[start[d[i]]], ov[start[d[i]]] = k[i], v[i]
                    start[d[i]] += 1
        k, v = ok, ov
    return v


def step_keys(sc):
    """The step's ordering keys of a scene's particles (make_key in aep_device.cuh)."""
    g = sc.grid
    x = sc.particles.positions
    res = np.asarray(g.resolution)
    cell = np.floor((x - g.min_bound) / g.h).astype(np.int64)
    cell = np.clip(cell, 0, res - 1)
    nb = ((res + 2) >> 2) + 2
    b, w = (cell + 3) >> 2, (cell + 3) & 3
    blk = (b[:, 2] * nb[1] + b[:, 1]) * nb[0] + b[:, 0]
    keys = (blk << 6) | (w[:, 2] << 4) | (w[:, 1] << 2) | w[:, 0]
    bits = int(np.ceil(np.log2(int(np.prod(nb)) * 64)))
    return keys.astype(np.uint32), bits


def test_tile_algorithm_is_a_stable_sort():
    rng = np.random.default_rng(0)
    for n, bits, hi in [(1, 3, 8), (4095, 9, 512), (4097, 8, 7), (9000, 17, 1 << 17), (12289, 22, 300)]:
        keys = rng.integers(0, hi, n)
        assert np.array_equal(tile_radix_sort(keys, bits), np.argsort(keys, kind="stable"))


def _gpu_sort(torch, keys, bits):
    lib = capi.load()
    n = len(keys)
    dev = torch.device("cuda", 0)
    k_in = torch.from_numpy(keys.astype(np.uint32).view(np.int32)).to(dev)
    v_in = torch.arange(n, dtype=torch.int32, device=dev)
    k_out = torch.empty_like(k_in)
    v_out = torch.empty_like(v_in)
    tb = lib.aep_sort_pairs_temp_bytes(n, bits)
    assert tb > 0
    tmp = torch.empty(tb, dtype=torch.uint8, device=dev)
    st = lib.aep_sort_pairs(k_in.data_ptr(), k_out.data_ptr(), v_in.data_ptr(), v_out.data_ptr(), n, bits,
                            tmp.data_ptr(), tb, None)
    torch.cuda.synchronize()
    assert st == capi.AEP_OK
    return k_out.cpu().numpy().view(np.uint32), v_out.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sand_column", "snow_sand_collision"])
def test_gpu_sort_of_step_keys_matches_stable_argsort(name):
    torch = pytest.importorskip("torch")
    sc = {"sand_column": scenes.sand_column, "snow_sand_collision": scenes.snow_sand_collision}[name]()
    keys, bits = step_keys(sc)
    for variant in ("as_generated", "nearly_sorted"):
        if variant == "nearly_sorted":  # the next ordering's input: sorted, a few changed
            keys = np.sort(keys)
            rng = np.random.default_rng(1)
            idx = rng.choice(len(keys), 20000, replace=False)
            keys[idx] = keys[rng.permutation(idx)]
        k, v = _gpu_sort(torch, keys, bits)
        want = np.argsort(keys, kind="stable")
        assert np.array_equal(v, want), (name, variant)
        assert np.array_equal(k, keys[want])


@pytest.mark.gpu
def test_gpu_sort_random_keys_every_width_and_size():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    for n, bits in [(1, 1), (5, 32), (4095, 7), (4096, 8), (4097, 9), (100003, 16), (300000, 25), (1 << 20, 32)]:
        for hi in (2, 1 << min(bits, 31)):  # many equal keys; all the bits
            keys = rng.integers(0, hi, n, dtype=np.int64).astype(np.uint32)
            if bits < 32:
                keys &= np.uint32((1 << bits) - 1)
            k, v = _gpu_sort(torch, keys, bits)
            want = np.argsort(keys, kind="stable")
            assert np.array_equal(v, want), (n, bits, hi)


def test_sort_argument_checks():
    lib = capi.load()
    assert lib.aep_sort_pairs_temp_bytes(-1, 8) == -1
    assert lib.aep_sort_pairs_temp_bytes(10, 0) == -1
    assert lib.aep_sort_pairs_temp_bytes(10, 33) == -1
    assert lib.aep_sort_pairs(None, None, None, None, 0, 8, None, 0, None) == capi.AEP_OK  # nothing to sort
    assert lib.aep_sort_pairs(None, None, None, None, 10, 8, None, 0, None) == capi.AEP_INVALID_ARG
