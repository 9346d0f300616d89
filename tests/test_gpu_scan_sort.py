"""The pipeline's device-wide prefix sum and radix sort (k_scan.cuh) against
numpy: exact equality at every size class the pipeline uses (one tile, tile
boundaries, the 432k-body batch, multi-million row counts), partial bit
ranges, 64-bit keys and stability among equal keys."""
import numpy as np
import pytest

from diomedes_gb300 import compute as C

pytestmark = pytest.mark.gpu


def _excl(a):
    a64 = a.astype(np.uint64)
    return (np.cumsum(a64) - a64).astype(np.uint32)  # wraps modulo 2**32


@pytest.mark.parametrize("n", [1, 2, 15, 4095, 4096, 4097, 65537, 432127, 2_000_003])
def test_scan_matches_cumsum(n):
    rng = np.random.default_rng(n)
    a = rng.integers(0, 64, n, dtype=np.uint32)
    a[rng.random(n) < 0.3] = 0
    out, total = C.device_exclusive_scan(a)
    assert np.array_equal(out, _excl(a))
    assert total == int(a.astype(np.uint64).sum()) % 2**32


def test_scan_wraps_modulo_2_32_and_repeats():
    rng = np.random.default_rng(7)
    a = rng.integers(0, 2**32, 300_001, dtype=np.uint64).astype(np.uint32)
    ref = _excl(a)
    # repeated launches on one look-back state (the epoch advances per launch)
    assert np.array_equal(C.device_exclusive_scan(a, repeats=7)[0], ref)


def test_empty_inputs():
    out, total = C.device_exclusive_scan(np.zeros(0, np.uint32))
    assert out.size == 0 and total == 0
    k, v = C.device_sort_pairs(np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    assert k.size == 0 and v.size == 0


def _check_sort(keys, begin, end):
    vals = np.arange(keys.size, dtype=np.uint32)
    ko, vo = C.device_sort_pairs(keys, vals, begin, end)
    width = end - begin
    digit = (keys.astype(np.uint64) >> np.uint64(begin))
    if width < 64:
        digit = digit & np.uint64((1 << width) - 1)
    order = np.argsort(digit, kind="stable")
    assert np.array_equal(vo, vals[order])
    assert np.array_equal(ko, keys[order])


@pytest.mark.parametrize("n,end", [(1, 32), (1000, 7), (8191, 17), (8192, 31), (8193, 32), (432127, 31),
                                   (1_500_001, 20)])
def test_sort_u32_matches_stable_argsort(n, end):
    rng = np.random.default_rng(n + end)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    _check_sort(keys, 0, end)


def test_sort_is_stable_among_equal_keys():
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 16, 200_003, dtype=np.uint32)  # long runs of equal keys
    _check_sort(keys, 0, 4)
    _check_sort(keys, 1, 3)


@pytest.mark.parametrize("n,begin,end", [(5, 0, 64), (100_000, 0, 64), (300_007, 8, 40), (4096 * 3 + 1, 0, 33)])
def test_sort_u64_matches_stable_argsort(n, begin, end):
    rng = np.random.default_rng(n)
    a = rng.integers(0, 50_000, n, dtype=np.uint64)
    b = rng.integers(0, 50_000, n, dtype=np.uint64)
    keys = (a << np.uint64(32)) | b  # row keys: (body a, body b)
    _check_sort(keys, begin, end)


def test_sort_of_already_sorted_and_reversed_keys():
    n = 100_000
    _check_sort(np.arange(n, dtype=np.uint32), 0, 17)
    _check_sort(np.arange(n, dtype=np.uint32)[::-1].copy(), 0, 17)


@pytest.mark.parametrize("n,live", [(864_000, 65_329), (864_000, 0), (5000, 4096), (5000, 4097), (4096, 9999)])
def test_scan_stops_at_the_device_count(n, live):
    rng = np.random.default_rng(live)
    a = rng.integers(0, 5, n, dtype=np.uint32)
    sentinel = np.full(n, 0xDEADBEEF, np.uint32)
    out, total = C.device_exclusive_scan(a, live=live, out=sentinel)
    m = min(live, n)
    assert np.array_equal(out[:m], _excl(a[:m]))
    assert (out[m:] == 0xDEADBEEF).all()  # past the live count: untouched
    assert total == int(a[:m].astype(np.uint64).sum())
