"""Properties the round kernel's swap-heap handling rests on, checked on the
CPU against the libstdc++ pop order of the reference's SwapPair heap
(oracle.swap_heap_order, reorder/swappair.h:112-120, reorder/reorder.h:
521-532).  No GPU is used here.

- A heap pops in non-increasing key order, so among the swaps whose two
  nodes are both unvisited the first one popped has the largest key; when
  no other qualifying swap shares that key, it can be read off the keys
  without the pops (the walk's shortcut).
- (l + r, r) packed in 12 + 12 bits orders like the 64-bit key
  ((l + r) << 32 | r + 2^31) for gains within +-2047 (the heap entries'
  direct keys).
- Replacing every key by its rank among the heap's keys (how many are
  smaller) leaves the pop order unchanged, ties included (the entries of
  heaps with larger gains)."""
import numpy as np
import pytest

import oracle


def _keys(lg, rg):
    return [(int(a) + int(b), int(b)) for a, b in zip(lg, rg)]


@pytest.mark.parametrize("M", [4, 8])
def test_first_unvisited_pop_is_the_unique_best_qualifying_swap(M):
    rng = np.random.default_rng(M)
    MM = M * M
    shortcuts = 0
    for t in range(3000):
        span = int(rng.choice([1, 2, 3, 6, 50]))
        lg = rng.integers(-span, span + 1, MM)
        rg = rng.integers(-span, span + 1, MM)
        order = oracle.swap_heap_order(lg, rg)
        vp = int(rng.integers(0, 1 << M)) & int(rng.integers(0, 1 << M))  # visited nodes of either side
        vt = int(rng.integers(0, 1 << M)) & int(rng.integers(0, 1 << M))
        ok = [not ((vp >> (x // M)) & 1) and not ((vt >> (x % M)) & 1) for x in range(MM)]
        if not any(ok):
            continue
        first = next(int(x) for x in order if ok[x])
        keys = _keys(lg, rg)
        best = max(keys[x] for x in range(MM) if ok[x])
        holders = [x for x in range(MM) if ok[x] and keys[x] == best]
        assert keys[first] == best  # pops never increase in key
        if len(holders) == 1:
            assert first == holders[0]
            shortcuts += 1
    assert shortcuts > 500  # the shortcut case is common, not vacuous


def test_packed_key_orders_like_the_64_bit_key():
    rng = np.random.default_rng(1)
    l = rng.integers(-1023, 1024, 20000)
    r = rng.integers(-1023, 1024, 20000)
    keep = (np.abs(l + r) <= 2047) & (np.abs(r) <= 2047)
    l, r = l[keep], r[keep]
    packed = ((l + r + 2048) << 12) | (r + 2048)
    wide = ((l + r).astype(np.int64) << 32) + (r.astype(np.int64) + (1 << 31))
    i, j = rng.integers(0, len(l), (2, 50000))
    assert np.array_equal(np.sign(packed[i] - packed[j]), np.sign(wide[i] - wide[j]))
    ends = np.array([-2047, 0, 2047])  # the range limits themselves
    for a in ends:
        for b in ends:
            assert 0 <= (a + 2048) < 4096 and 0 <= (b + 2048) < 4096


@pytest.mark.parametrize("M", [4, 8])
def test_ranked_keys_give_the_same_pop_order(M):
    rng = np.random.default_rng(10 + M)
    MM = M * M
    for t in range(2000):
        span = int(rng.choice([1, 2, 4, 3000]))
        lg = rng.integers(-span, span + 1, MM)
        rg = rng.integers(-span, span + 1, MM)
        keys = _keys(lg, rg)
        rank = np.array([sum(1 for y in keys if y < x) for x in keys], np.int32)
        # a key of (rank, 0) orders the swaps by rank alone
        assert np.array_equal(oracle.swap_heap_order(rank, np.zeros(MM, np.int32)), oracle.swap_heap_order(lg, rg))
