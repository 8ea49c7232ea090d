"""CPU: the GPU engine's host-side type model (constructors, normalising shortcuts,
size/extent/true extent, iov_len) agrees with the oracle on seeded random types and on
the reference's own bounds known-answers (test/simple/lbub.c)."""
import pytest

import yaksa_gb300 as yk
from typegen import BASE, Gen, build


@pytest.mark.parametrize("seed", range(40))
def test_random_type_bounds_match_oracle(prod, oracle, seed):
    base = sorted(BASE)[seed % len(BASE)]
    g = Gen(oracle, seed, max_depth=3)
    for _ in range(10):
        r = g.gen(base)
        kp, ko = [], []
        hp, ho = build(prod, r, kp), build(oracle, r, ko)
        assert prod.size(hp) == oracle.size(ho), r
        assert prod.extent(hp) == oracle.extent(ho), r
        assert prod.true_extent(hp) == oracle.true_extent(ho), r
        assert prod.iov_len(3, hp) == oracle.iov_len(3, ho), r
        for y, keep in ((prod, kp), (oracle, ko)):
            for h in reversed(keep):
                y.type_free(h)
    g.free()


def test_lbub_known_answers(prod):
    """Values asserted by the reference's test/simple/lbub.c:45-80."""
    y = prod
    tmp = y.type_create_contig(4, yk.TYPE_BYTE)
    evil = y.type_create_resized(tmp, -3, 9)
    assert y.size(evil) == 4
    assert y.extent(evil) == (-3, 9)
    assert y.true_extent(evil) == (0, 4)
    c3 = y.type_create_contig(3, evil)
    assert y.size(c3) == 12
    assert y.extent(c3) == (-3, 27)
    assert y.true_extent(c3) == (0, 22)
    for h in (c3, evil, tmp):
        y.type_free(h)


def test_normalising_shortcuts(prod, oracle):
    for y in (prod, oracle):
        # struct of identical child types becomes hindexed: no alignment padding
        s = y.type_create_struct([1, 1], [0, 4], [yk.TYPE_INT32_T, yk.TYPE_INT32_T])
        assert y.extent(s) == (0, 8)
        # struct of mixed types pads ub to the largest alignment (yaksa_struct.c:95-101)
        m = y.type_create_struct([1, 1], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT])
        assert y.size(m) == 12 and y.extent(m) == (0, 16)
        # blkhindx whose displacements are a progression from 0 behaves as hvector
        b = y.type_create_hindexed_block(2, [0, 16, 32, 48], yk.TYPE_FLOAT)
        assert y.size(b) == 32 and y.extent(b) == (0, 56)
        for h in (s, m, b):
            y.type_free(h)


def test_null_results(prod):
    assert prod.type_create_contig(0, yk.TYPE_INT) == yk.TYPE_NULL
    assert prod.type_create_hindexed([0, 0], [0, 4], yk.TYPE_INT) == yk.TYPE_NULL
    assert prod.size(yk.TYPE_NULL) == 0


def test_pair_type_bounds(prod, oracle):
    for h in (yk.TYPE_FLOAT_INT, yk.TYPE_DOUBLE_INT, yk.TYPE_SHORT_INT, yk.TYPE_2INT,
              yk.TYPE_LONG_INT, yk.TYPE_C_COMPLEX, yk.TYPE_C_DOUBLE_COMPLEX):
        assert prod.size(h) == oracle.size(h)
        assert prod.extent(h) == oracle.extent(h)
        assert prod.true_extent(h) == oracle.true_extent(h)
    assert prod.size(yk.TYPE_SHORT_INT) == 6 and prod.extent(yk.TYPE_SHORT_INT) == (0, 8)
