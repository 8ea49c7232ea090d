"""GPU: edge cases of the pack/unpack boundary, each compared with the oracle: empty
requests (count 0, zero budget, offset at or past the end), budgets smaller than one
builtin, ragged unpack sizes, the NULL type, zero-length blocks, negative strides and
negative extents.

Tolerance: byte-identical.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import dev_copy, fill, host_of
from typegen import footprint

pytestmark = pytest.mark.gpu


def both(prod, oracle, mk):
    return mk(prod), mk(oracle)


def run_pair(cuda, prod, oracle, tp, to, count, base, offset, nbytes, direction, span, lo):
    rng = np.random.default_rng(offset + nbytes + count)
    typed = fill(rng, span + 64, base)
    packed = fill(rng, max(nbytes, 1) + 64, base)
    tg, pg = dev_copy(cuda, typed), dev_copy(cuda, packed)
    th, ph = typed.copy(), packed.copy()
    if direction == "pack":
        ap = prod.pack(tg.data_ptr() + 32 - lo, count, tp, offset, pg.data_ptr(), nbytes)
        ao = oracle.pack(th.ctypes.data + 32 - lo, count, to, offset, ph.ctypes.data, nbytes)
    else:
        ap = prod.unpack(pg.data_ptr(), nbytes, tg.data_ptr() + 32 - lo, count, tp, offset)
        ao = oracle.unpack(ph.ctypes.data, nbytes, th.ctypes.data + 32 - lo, count, to, offset)
    cuda.cuda.synchronize()
    assert ap == ao, (direction, offset, nbytes, ap, ao)
    assert np.array_equal(host_of(cuda, tg), th)
    assert np.array_equal(host_of(cuda, pg), ph)
    return ap


def test_empty_and_clipped_requests(cuda, prod, oracle):
    tp, to = both(prod, oracle, lambda y: y.type_create_hvector(7, 3, 40, yk.TYPE_INT32_T))
    size, ext = prod.size(tp), prod.extent(tp)[1]
    span = 3 * ext
    for direction in ("pack", "unpack"):
        assert run_pair(cuda, prod, oracle, tp, to, 0, "int32", 0, 64, direction, span, 0) == 0
        assert run_pair(cuda, prod, oracle, tp, to, 3, "int32", 0, 0, direction, span, 0) == 0
        assert run_pair(cuda, prod, oracle, tp, to, 3, "int32", 3 * size, 64, direction, span, 0) == 0
        # a budget smaller than one builtin moves nothing; a ragged one stops on a builtin
        assert run_pair(cuda, prod, oracle, tp, to, 3, "int32", 8, 3, direction, span, 0) == 0
        assert run_pair(cuda, prod, oracle, tp, to, 3, "int32", 8, 30, direction, span, 0) == 28
        # offset near the end, budget past it
        assert run_pair(cuda, prod, oracle, tp, to, 3, "int32", 3 * size - 12, 100, direction, span,
                        0) == 12
    prod.type_free(tp)
    oracle.type_free(to)


def test_null_type(cuda, prod, oracle):
    buf = cuda.zeros(16, dtype=cuda.uint8, device="cuda")
    for y in (prod, oracle):
        assert y.size(yk.TYPE_NULL) == 0
    assert prod.pack(buf.data_ptr(), 4, yk.TYPE_NULL, 0, buf.data_ptr(), 16) == 0
    assert prod.unpack(buf.data_ptr(), 16, buf.data_ptr(), 4, yk.TYPE_NULL, 0) == 0


@pytest.mark.parametrize("direction", ["pack", "unpack"])
def test_zero_length_blocks_and_negative_layouts(cuda, prod, oracle, direction):
    cases = [
        # hindexed with empty blocks between non-empty ones
        (lambda y: y.type_create_hindexed([0, 3, 0, 0, 5, 1, 0], [0, 8, 40, 40, 64, 100, 120],
                                          yk.TYPE_INT32_T), "int32"),
        # negative stride
        (lambda y: y.type_create_hvector(9, 2, -24, yk.TYPE_DOUBLE), "double"),
        # negative extent (elements laid out downwards)
        (lambda y: y.type_create_resized(y.type_create_contig(3, yk.TYPE_FLOAT), 0, -16), "float"),
        # struct with an empty member
        (lambda y: y.type_create_struct([2, 0, 1], [0, 8, 24], [yk.TYPE_INT16_T, yk.TYPE_DOUBLE,
                                                                 yk.TYPE_INT64_T]), "int8"),
    ]
    for mk, base in cases:
        tp, to = both(prod, oracle, mk)
        for count in (1, 4):
            lo, hi, size = footprint(oracle, to, count)
            total = size * count
            for off, n in ((0, total), (size, total), (0, total // 2 + 1)):
                run_pair(cuda, prod, oracle, tp, to, count, base, off, n, direction, hi - lo, lo)
        prod.type_free(tp)
        oracle.type_free(to)


@pytest.mark.parametrize("nranks", [2, 3, 8])
def test_shard_parts_on_gpu(cuda, prod, oracle, nranks):
    """The parts yaksa_gb300_shard gives, each packed by the product on its own, make up
    the oracle's one-call pack; unpacked part by part they give its one-call unpack."""
    from helpers import Pair
    from typegen import Gen
    g = Gen(oracle, 15000 + nranks, max_depth=3)
    rng = np.random.default_rng(nranks)
    for i in range(8):
        base = ["int32", "double", "int8", "float"][i % 4]
        pair = Pair(prod, oracle, g.gen(base))
        count = int(rng.integers(1, 7))
        lo, hi, size = footprint(oracle, pair.ho, count)
        total = size * count
        typed = fill(rng, hi - lo + 64, base)
        tg = dev_copy(cuda, typed)
        exp = np.zeros(total + 16, dtype=np.uint8)
        oracle.pack(typed.ctypes.data + 32 - lo, count, pair.ho, 0, exp.ctypes.data, total)
        pg = cuda.zeros(total + 16, dtype=cuda.uint8, device="cuda")
        parts = [prod.shard(pair.hp, count, r, nranks) for r in range(nranks)]
        assert sum(n for _, n in parts) == total
        for off, n in parts:
            assert prod.pack(tg.data_ptr() + 32 - lo, count, pair.hp, off, pg.data_ptr() + off, n) == n
        cuda.cuda.synchronize()
        assert np.array_equal(host_of(cuda, pg)[:total], exp[:total])
        # unpack the parts into a fresh buffer, in reverse order (no order between parts)
        dst = fill(rng, hi - lo + 64, base)
        dg, d_o = dev_copy(cuda, dst), dst.copy()
        oracle.unpack(exp.ctypes.data, total, d_o.ctypes.data + 32 - lo, count, pair.ho, 0)
        pe = dev_copy(cuda, exp)
        for off, n in reversed(parts):
            assert prod.unpack(pe.data_ptr() + off, n, dg.data_ptr() + 32 - lo, count, pair.hp, off) == n
        cuda.cuda.synchronize()
        ok = np.array_equal(host_of(cuda, dg), d_o)
        offs = np.empty(total, dtype=np.int64)
        f = oracle.lib.yaksa_oracle_byte_offsets
        import ctypes
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p]
        assert f(pair.ho, count, offs.ctypes.data) == 0
        if len(np.unique(offs)) == total:       # no byte reached twice: order is free
            assert ok
        pair.free()
    g.free()
