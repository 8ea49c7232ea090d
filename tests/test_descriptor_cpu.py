"""CPU: the address every GPU work unit will touch equals the oracle's typemap.

yaksa_gb300_debug_locate runs the kernels' decomposition (yk_locate.h: level chain,
Granlund-Montgomery division, table searches) on the CPU over the same descriptor the
GPU receives.  For seeded random types, every packed byte's typed-side offset must
equal the offset the oracle's typemap walk assigns to it.  This also proves every
address lies inside the buffer footprint before any kernel runs on a GPU.
"""
import ctypes

import numpy as np
import pytest

import yaksa_gb300 as yk
from typegen import BASE, Gen, build, footprint


def locate(prod, h, count, typed, pos):
    pos = np.ascontiguousarray(pos, dtype=np.uint64)
    off = np.empty(len(pos), dtype=np.int64)
    f = prod.lib.yaksa_gb300_debug_locate
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p,
                  ctypes.c_void_p]
    rc = f(h, count, typed, len(pos), pos.ctypes.data, off.ctypes.data)
    assert rc == 0, rc
    return off


def typemap(oracle, h, count):
    size = oracle.size(h)
    out = np.empty(size * count, dtype=np.int64)
    f = oracle.lib.yaksa_oracle_byte_offsets
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p]
    assert f(h, count, out.ctypes.data) == 0
    return out


BASES = ["int8", "int16", "int32", "int64", "float", "double", "c_complex", "c_double_complex",
         "short_int", "double_int", "float_int", "2int", "bool"]


@pytest.mark.parametrize("seed", range(60))
def test_every_byte_offset_matches_oracle(prod, oracle, seed):
    base = BASES[seed % len(BASES)]
    g = Gen(oracle, 5000 + seed, max_depth=3 + seed % 2)
    for i in range(8):
        r = g.gen(base)
        kp, ko = [], []
        hp, ho = build(prod, r, kp), build(oracle, r, ko)
        count = 1 + (i % 3)
        expect = typemap(oracle, ho, count)
        pos = np.arange(len(expect), dtype=np.uint64)
        lo, hi, _ = footprint(oracle, ho, count)
        for typed in (0, 1):
            got = locate(prod, hp, count, typed, pos)
            bad = np.nonzero(got != expect)[0]
            assert len(bad) == 0, (r, count, typed, bad[:5], got[bad[:5]], expect[bad[:5]])
            assert got.min() >= lo and got.max() < hi
        for y, keep in ((prod, kp), (oracle, ko)):
            for h in reversed(keep):
                y.type_free(h)
    g.free()


def test_large_counts_use_64bit_positions(prod, oracle):
    """Positions beyond 2^32 take the 64-bit decomposition; spot-check them."""
    t_p = prod.type_create_hvector(3, 5, 48, yk.TYPE_DOUBLE)
    t_o = oracle.type_create_hvector(3, 5, 48, yk.TYPE_DOUBLE)
    size = prod.size(t_p)
    count = (1 << 33) // size + 7
    rng = np.random.default_rng(3)
    pos = np.sort(rng.integers(0, count * size, 4000)).astype(np.uint64)
    got = locate(prod, t_p, count, 0, pos)
    # closed form: element e = p // size, within-element from the oracle's map of one element
    one = typemap(oracle, t_o, 1)
    lb, ext = oracle.extent(t_o)
    e = pos // size
    exp = e.astype(np.int64) * ext + one[(pos % size).astype(np.int64)]
    assert np.array_equal(got, exp)
    prod.type_free(t_p)
    oracle.type_free(t_o)


def test_benchmark_shapes(prod, oracle):
    """The benchmark configurations' types, at reduced sizes."""
    shapes = []
    for sub, st in (([64, 64, 2], [0, 0, 0]), ([64, 64, 2], [0, 0, 62]), ([64, 2, 64], [0, 62, 0]),
                    ([2, 64, 64], [62, 0, 0])):
        shapes.append(lambda y, sub=sub, st=st: y.type_create_subarray([64, 64, 64], sub, st,
                                                                       yk.SUBARRAY_ORDER_C,
                                                                       yk.TYPE_FLOAT))
    shapes.append(lambda y: y.type_create_hvector(1024, 4, 128, yk.TYPE_DOUBLE))

    def struct_(y):
        s = y.type_create_struct([1, 3], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT])
        return y.type_create_resized(s, 0, 32)
    shapes.append(struct_)
    rng = np.random.default_rng(5)
    blens = np.clip(np.round(np.exp(np.log(16) + rng.standard_normal(512))), 1, 4096).astype(np.int64)
    displs = np.cumsum(blens * 4 + 4 * rng.integers(0, 8, 512)) - blens * 4
    rng.shuffle(displs)
    shapes.append(lambda y: y.type_create_hindexed(blens.tolist(), displs.tolist(), yk.TYPE_INT32_T))
    offs = np.sort(rng.integers(0, 4000, 512))
    shapes.append(lambda y: y.type_create_indexed_block(8, offs.tolist(), yk.TYPE_DOUBLE))
    for mk in shapes:
        hp, ho = mk(prod), mk(oracle)
        for count in (1, 2):
            expect = typemap(oracle, ho, count)
            for typed in (0, 1):
                got = locate(prod, hp, count, typed, np.arange(len(expect)))
                assert np.array_equal(got, expect)


@pytest.mark.parametrize("nblk,zero_frac,count", [(1 << 14, 0.0, 1), (5000, 0.3, 2), (3, 0.0, 3),
                                                  (1 << 12, 0.5, 1)])
def test_hindexed_tile_table(prod, oracle, nblk, zero_frac, count):
    """Lognormal block lengths (the irregular config's distribution, fewer blocks),
    with empty blocks mixed in: every byte's address matches the oracle."""
    rng = np.random.default_rng(nblk)
    blens = np.clip(np.round(np.exp(np.log(16) + rng.standard_normal(nblk))), 1, 4096).astype(np.int64)
    blens[rng.random(nblk) < zero_frac] = 0
    if blens.sum() == 0:
        blens[0] = 3
    slots = rng.permutation(nblk)
    gaps = rng.integers(0, 4, nblk)
    starts = np.cumsum(blens[slots] + gaps) - blens[slots]
    displs = np.empty(nblk, dtype=np.int64)
    displs[slots] = starts * 4
    hp = prod.type_create_hindexed(blens.tolist(), displs.tolist(), yk.TYPE_INT32_T)
    ho = oracle.type_create_hindexed(blens.tolist(), displs.tolist(), yk.TYPE_INT32_T)
    expect = typemap(oracle, ho, count)
    got = locate(prod, hp, count, 0, np.arange(len(expect)))
    assert np.array_equal(got, expect)
    prod.type_free(hp)
    oracle.type_free(ho)


def desc_info(prod, h, typed):
    f = prod.lib.yaksa_gb300_debug_desc_info
    f.restype = ctypes.c_int
    vals = [ctypes.c_int() for _ in range(5)]
    assert f(ctypes.c_uint64(h), typed, *[ctypes.byref(v) for v in vals]) == 0
    return dict(zip(["vec_align", "unit", "may_overlap", "sorted_blocks", "nlev"],
                    [v.value for v in vals]))


@pytest.mark.parametrize("seed", range(40))
def test_vector_units_and_overlap_flag(prod, oracle, seed):
    """Every vec_align-byte unit of the packed stream maps to vec_align contiguous,
    vec_align-aligned typed bytes; a typemap that reaches a byte twice is flagged."""
    base = BASES[seed % len(BASES)]
    g = Gen(oracle, 7000 + seed, max_depth=3, overlap=bool(seed % 2))
    for i in range(8):
        r = g.gen(base)
        kp, ko = [], []
        hp, ho = build(prod, r, kp), build(oracle, r, ko)
        expect = typemap(oracle, ho, 1)
        info = desc_info(prod, hp, 0)
        va = info["vec_align"]
        if len(expect) % va == 0:
            units = expect.reshape(-1, va)
            assert np.all(units[:, 0] % va == 0), (r, va)
            assert np.all(units - units[:, :1] == np.arange(va)), (r, va)
        dup = len(np.unique(expect)) != len(expect)
        if dup:
            assert info["may_overlap"], r
            assert desc_info(prod, hp, 1)["may_overlap"], r
        for y, keep in ((prod, kp), (oracle, ko)):
            for h in reversed(keep):
                y.type_free(h)
    g.free()


def d32_info(prod, h, typed=1):
    f = prod.lib.yaksa_gb300_debug_d32
    f.restype = ctypes.c_int
    bits, d32 = ctypes.c_int(), ctypes.c_int()
    assert f(ctypes.c_uint64(h), typed, ctypes.byref(bits), ctypes.byref(d32)) == 0
    return bits.value, d32.value


@pytest.mark.parametrize("case,expect", [("small_sorted", (3, 1)), ("small_unsorted", (3, 0)),
                                         ("offset_over", (1, 0)), ("table_over", (0, 0)),
                                         ("negative", (3, 1))])
def test_32bit_forms_at_the_limits(prod, case, expect):
    """The descriptor's 32-bit forms at the edges of 32 bits, for overlapping blocks of 8
    int32 (32 bytes): bit 1 (a 32-bit copy of the displacements), bit 2 (every
    displacement plus the block fits too) and the sorted-block 32-bit-offset flag.  Byte
    displacements near 0, in ascending or shuffled order; near 2^31 with one block
    reaching past 2^31 - 1 (the table fits, the offsets do not); one displacement of 2^31
    (no 32-bit table); and from -2^31 up."""
    rng = np.random.default_rng(len(case))
    start = {"small_sorted": 0, "small_unsorted": 0, "offset_over": (1 << 31) - 64 - 4096,
             "table_over": (1 << 31) - 64 - 4096, "negative": -(1 << 31)}[case]
    offs = np.sort(start + rng.integers(0, 1024, 300) * 4)
    if case == "small_unsorted":
        rng.shuffle(offs)
    elif case == "offset_over":
        offs = np.append(offs, (1 << 31) - 16)      # its last element ends at 2^31 + 15
    elif case == "table_over":
        offs = np.append(offs, 1 << 31)
    h = prod.type_create_hindexed_block(8, offs.tolist(), yk.TYPE_INT32_T)
    assert desc_info(prod, h, 1)["may_overlap"]
    assert d32_info(prod, h) == expect
    prod.type_free(h)
