"""GPU: the benchmark configurations, bit-exact against the oracle.

Each config keeps its shape and value distribution at a size the oracle checks in
seconds: the 1024x16 hvector of doubles (full size), halo faces of a 128^3 float grid,
hindexed int32 with lognormal block lengths, the {int64, float x3} struct resized to
32 bytes, and indexed_block unpacks with SUM/MAX/BXOR/PROD over overlapping sorted
blocks.  Tolerance: byte-identical.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import assert_same_bytes, dev_copy, host_of

pytestmark = pytest.mark.gpu


def both(prod, oracle, mk):
    return mk(prod), mk(oracle)


def check_roundtrip(cuda, prod, oracle, tp, to, count, typed, packed0, op=yk.OP_REPLACE,
                    directions=("pack", "unpack"), what=""):
    size = oracle.size(to)
    P = size * count
    for d in directions:
        th, ph = typed.copy(), packed0.copy()
        tg, pg = dev_copy(cuda, typed), dev_copy(cuda, packed0)
        if d == "pack":
            ao = oracle.pack(th.ctypes.data, count, to, 0, ph.ctypes.data, P, op=op)
            ag = prod.pack(tg.data_ptr(), count, tp, 0, pg.data_ptr(), P, op=op)
        else:
            ao = oracle.unpack(ph.ctypes.data, P, th.ctypes.data, count, to, 0, op=op)
            ag = prod.unpack(pg.data_ptr(), P, tg.data_ptr(), count, tp, 0, op=op)
        assert ao == ag == P
        assert_same_bytes(host_of(cuda, pg), ph, f"{what} {d} packed")
        assert_same_bytes(host_of(cuda, tg), th, f"{what} {d} typed")


def test_hvector_double_full_size(cuda, prod, oracle):
    rng = np.random.default_rng(0)
    tp, to = both(prod, oracle, lambda L: L.type_create_hvector(1024, 4, 128, yk.TYPE_DOUBLE))
    a = rng.uniform(-1, 1, 1024 * 16).view(np.uint8)
    check_roundtrip(cuda, prod, oracle, tp, to, 1, a, np.zeros(32768, np.uint8), what="hvector")


@pytest.mark.parametrize("face", range(6))
def test_halo_faces(cuda, prod, oracle, face):
    n = 128
    specs = [([n, n, 2], [0, 0, 0]), ([n, n, 2], [0, 0, n - 2]), ([n, 2, n], [0, 0, 0]),
             ([n, 2, n], [0, n - 2, 0]), ([2, n, n], [0, 0, 0]), ([2, n, n], [n - 2, 0, 0])]
    sub, st = specs[face]
    tp, to = both(prod, oracle, lambda L: L.type_create_subarray([n] * 3, sub, st,
                                                                 yk.SUBARRAY_ORDER_C, yk.TYPE_FLOAT))
    rng = np.random.default_rng(face)
    g = rng.uniform(-1, 1, n ** 3).astype(np.float32).view(np.uint8)
    check_roundtrip(cuda, prod, oracle, tp, to, 1, g, np.zeros(2 * n * n * 4, np.uint8), what="face")


@pytest.mark.parametrize("nb", [1 << 12, 1 << 16])
def test_hindexed_lognormal(cuda, prod, oracle, nb):
    rng = np.random.default_rng(nb)
    blens = np.clip(np.round(np.exp(np.log(16) + rng.standard_normal(nb))), 1, 4096).astype(np.int64)
    total_slots = int(blens.sum()) * 4
    gaps = rng.integers(0, 2 * (total_slots - int(blens.sum())) // nb + 1, nb)
    order = rng.permutation(nb)
    starts = np.cumsum(blens[order] + gaps) - blens[order]
    displs = np.empty(nb, dtype=np.int64)
    displs[order] = starts * 4
    ext = int((starts[-1] + blens[order][-1]) * 4 + 64)

    def mk(L):
        h = L.type_create_hindexed_arrays(nb, blens.ctypes.data, displs.ctypes.data, yk.TYPE_INT32_T)
        r = L.type_create_resized(h, 0, ext)
        L.type_free(h)
        return r
    tp, to = both(prod, oracle, mk)
    typed = rng.integers(0, 256, ext, dtype=np.uint8)
    packed = rng.integers(0, 256, int(blens.sum()) * 4, dtype=np.uint8)
    check_roundtrip(cuda, prod, oracle, tp, to, 1, typed, packed, what="hindexed")
    # and two elements back to back
    typed2 = rng.integers(0, 256, 2 * ext, dtype=np.uint8)
    check_roundtrip(cuda, prod, oracle, tp, to, 2, typed2, np.concatenate([packed, packed]),
                    what="hindexed x2")


@pytest.mark.parametrize("op", [yk.OP_REPLACE, yk.OP_SUM, yk.OP_MAX])
def test_struct_int64_float3(cuda, prod, oracle, op):
    def mk(L):
        s = L.type_create_struct([1, 3], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT])
        r = L.type_create_resized(s, 0, 32)
        L.type_free(s)
        return r
    tp, to = both(prod, oracle, mk)
    count = 1 << 16
    rng = np.random.default_rng(op)
    typed = rng.uniform(-1, 1, count * 8).astype(np.float32).view(np.uint8)
    packed = rng.uniform(-1, 1, count * 5).astype(np.float32).view(np.uint8)
    check_roundtrip(cuda, prod, oracle, tp, to, count, typed, packed, op=op, what=f"struct op{op}")


@pytest.mark.parametrize("base,h,es,op", [("double", yk.TYPE_DOUBLE, 8, yk.OP_SUM),
                                          ("int64", yk.TYPE_INT64_T, 8, yk.OP_MAX),
                                          ("uint32", yk.TYPE_UINT32_T, 4, yk.OP_BXOR),
                                          ("c_complex", yk.TYPE_C_COMPLEX, 8, yk.OP_PROD)])
def test_reduction_overlapping_sorted_blocks(cuda, prod, oracle, base, h, es, op):
    nblk = 1 << 16
    nel = nblk * 8
    rng = np.random.default_rng(es + op)
    offs = np.sort(rng.integers(0, nel - 8, nblk)).astype(np.int64)
    tp, to = both(prod, oracle, lambda L: L.type_create_indexed_block_array(nblk, 8, offs.ctypes.data, h))
    if base == "double":
        target, packed = rng.standard_normal(nel), rng.standard_normal(nel)
    elif base == "int64":
        target = rng.integers(-(1 << 63), (1 << 63) - 1, nel, dtype=np.int64)
        packed = rng.integers(-(1 << 63), (1 << 63) - 1, nel, dtype=np.int64)
    elif base == "uint32":
        target = rng.integers(0, 1 << 32, nel, dtype=np.uint64).astype(np.uint32)
        packed = rng.integers(0, 1 << 32, nel, dtype=np.uint64).astype(np.uint32)
    else:
        def z(n):
            return (np.exp(rng.uniform(np.log(0.9), np.log(1.1), n)) *
                    np.exp(1j * rng.uniform(0, 2 * np.pi, n))).astype(np.complex64)
        target, packed = z(nel), z(nel)
    check_roundtrip(cuda, prod, oracle, tp, to, 1, target.view(np.uint8), packed.view(np.uint8),
                    op=op, directions=("unpack",), what=f"reduce {base}")
