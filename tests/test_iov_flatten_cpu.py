"""CPU: segment lists (yaksa_iov, yaksa_iov_len, yaksa_iov_len_max) and flattened types
(yaksa_flatten_size, yaksa_flatten, yaksa_unflatten) of the product against the oracle
on seeded random types.

The product's segment list is host code, so these run without a GPU.  Two independent
checks per type: the list equals the oracle's entry for entry (the oracle restates the
reference recursion, src/frontend/iov/yaksa_iov.c:48-359), and the pieces laid end to
end are exactly the oracle's typemap.  A flattened-and-unflattened type must keep its
bounds, its segment list and every byte offset of its typemap.  The reference's own
iov test (test/iov/iov.c) also runs against the product library over the reference's
test matrix (oracle/run_reftests.py; record in tests/golden/reftests_oracle.txt).
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import Pair
from test_descriptor_cpu import BASES, locate, typemap
from typegen import Gen

BUF = 1 << 40   # base address of the lists: the walk adds offsets to it, never reads it


def listing(y, count, h, offset, max_len):
    try:
        return y.iov(BUF, count, h, offset, max_len)
    except yk.YaksaError as e:
        return ("error", e.rc)


@pytest.mark.parametrize("seed", range(24))
def test_iov_matches_oracle_and_typemap(prod, oracle, seed):
    rng = np.random.default_rng(seed)
    base = BASES[seed % len(BASES)]
    g = Gen(oracle, 3000 + seed, max_depth=3)
    for i in range(6):
        pair = Pair(prod, oracle, g.gen(base))
        count = int(rng.integers(1, 4))
        n = prod.iov_len(count, pair.hp)
        assert n == oracle.iov_len(count, pair.ho)
        full = listing(prod, count, pair.hp, 0, n)
        assert full == listing(oracle, count, pair.ho, 0, n)
        assert len(full) == n
        # the pieces in order are the typemap
        offs = np.concatenate([np.arange(a - BUF, a - BUF + ln) for a, ln in full if ln] or
                              [np.empty(0, dtype=np.int64)])
        assert np.array_equal(offs, typemap(oracle, pair.ho, count))
        # partial lists from an offset, with room for part of the rest
        for _ in range(6):
            off = int(rng.integers(0, n + 1))
            mx = int(rng.integers(0, n + 2))
            assert listing(prod, count, pair.hp, off, mx) == listing(oracle, count, pair.ho, off, mx)
        # leading pieces that fit in a byte budget
        total = prod.size(pair.hp) * count
        for mb in [0, total, total + 7] + [int(x) for x in rng.integers(0, total + 1, 6)]:
            assert prod.iov_len_max(count, pair.hp, mb) == oracle.iov_len_max(count, pair.ho, mb), mb
        pair.free()
    g.free()


def test_iov_len_max_is_a_prefix_of_the_list(prod):
    """The count and bytes iov_len_max reports are those of the list's leading pieces."""
    t = prod.type_create_hindexed([3, 0, 5, 2, 7], [0, 40, 80, 200, 300], yk.TYPE_INT32_T)
    full = prod.iov(BUF, 2, t, 0, prod.iov_len(2, t))
    for mb in range(0, 2 * prod.size(t) + 9):
        n, b = prod.iov_len_max(2, t, mb)
        assert b == sum(ln for _, ln in full[:n]) <= mb
        assert n == len(full) or b + full[n][1] > mb
    prod.type_free(t)


def test_pair_pieces_are_never_split(prod, oracle):
    """short_int has two pieces per element: lists and budgets take them in pairs."""
    for y in (prod, oracle):
        t = y.type_create_contig(4, yk.TYPE_SHORT_INT)
        assert y.iov_len(3, t) == 24
        assert len(y.iov(BUF, 3, t, 0, 5)) == 4
        assert y.iov_len_max(3, t, 6 + 5) == (2, 6)
        y.type_free(t)


def test_contiguous_type_is_one_piece_whatever_the_offset(prod, oracle):
    for y in (prod, oracle):
        t = y.type_create_contig(10, yk.TYPE_DOUBLE)
        assert y.iov(BUF, 3, t, 0, 4) == [(BUF, 240)]
        assert y.iov(BUF, 3, t, 5, 4) == [(BUF, 240)]
        assert y.iov(BUF, 3, t, 0, 0) == []
        y.type_free(t)


@pytest.mark.parametrize("seed", range(24))
def test_flatten_roundtrip(prod, oracle, seed):
    rng = np.random.default_rng(seed)
    base = BASES[seed % len(BASES)]
    g = Gen(oracle, 4000 + seed, max_depth=3)
    for i in range(5):
        pair = Pair(prod, oracle, g.gen(base))
        data = prod.flatten(pair.hp)
        u = prod.unflatten(data)
        assert prod.size(u) == prod.size(pair.hp)
        assert prod.extent(u) == prod.extent(pair.hp)
        assert prod.true_extent(u) == prod.true_extent(pair.hp)
        count = int(rng.integers(1, 4))
        n = prod.iov_len(count, u)
        assert n == prod.iov_len(count, pair.hp)
        assert prod.iov(BUF, count, u, 0, n) == prod.iov(BUF, count, pair.hp, 0, n)
        expect = typemap(oracle, pair.ho, count)
        pos = np.arange(len(expect), dtype=np.uint64)
        for typed in (0, 1):
            assert np.array_equal(locate(prod, u, count, typed, pos), expect)
        # a flattened copy flattens to the same bytes
        assert prod.flatten(u) == data
        prod.type_free(u)
        pair.free()
    g.free()


def test_unflatten_builtin_and_rejects_garbage(prod):
    u = prod.unflatten(prod.flatten(yk.TYPE_DOUBLE))
    assert prod.size(u) == 8 and prod.extent(u) == (0, 8)
    prod.type_free(u)
    with pytest.raises(yk.YaksaError):
        prod.unflatten(b"\0" * 256)
