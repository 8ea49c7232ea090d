"""GPU: unpacks into overlapping targets under SUM, MAX, MIN, BAND, BOR and BXOR on 4- and
8-byte integers, folded in by L2 reductions (yk_red_kernel), against the oracle.

The reference applies the blocks of an unpack in block order, element by element
(src/backend/seq/genpup.py:119-211, operators :302-327); for these operators the result
does not depend on that order, so the reduction form must give the same bytes whatever
order the L2 applies them in.  Cases: sorted and unsorted block offsets with heavy
overlap (many blocks on the same elements), block lengths that are and are not powers
of two, the packed range cut into segments on element boundaries, uint32 handles (which
alias the signed types, so MAX/MIN compare signed), and the library's own launch
counter showing the form ran.  Operators outside the set (PROD, LAND), 2-byte integers,
floating point and a typed buffer off the element size keep the ordered kernels; every
case matches the oracle and the form switched off.  Tolerance: byte-identical.
"""
import ctypes

import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import assert_same_bytes, dev_copy, fill, host_of, segments

pytestmark = pytest.mark.gpu

RED_OPS = [yk.OP_SUM, yk.OP_MAX, yk.OP_MIN, yk.OP_BAND, yk.OP_BOR, yk.OP_BXOR]
INT_TYPES = [("int32", yk.TYPE_INT32_T, 4), ("uint32", yk.TYPE_UINT32_T, 4),
             ("int64", yk.TYPE_INT64_T, 8)]


def red_launches(prod, mode=-1):
    n = ctypes.c_ulonglong(0)
    assert prod.lib.yaksa_gb300_debug_l2_reduce(mode, ctypes.byref(n)) == 0
    return n.value


def unpack_case(cuda, prod, oracle, ctor, args, base_h, es, op, seed, nseg=1, shift=0,
                base="int32"):
    """Unpack random packed data into a random target through the type on both
    libraries (nseg segments on element boundaries); returns the red launches used."""
    tp, to = getattr(prod, ctor)(*args, base_h), getattr(oracle, ctor)(*args, base_h)
    rng = np.random.default_rng(seed)
    lo, text = oracle.true_extent(to)
    P = oracle.size(to)
    pad = 64
    typed0 = fill(rng, text + 2 * pad, base)
    packed0 = fill(rng, P, base)
    t_o, t_p = typed0.copy(), dev_copy(cuda, typed0)
    p_p = dev_copy(cuda, packed0)
    before = red_launches(prod)
    for s, n in segments(rng, P, es, nseg):
        ao = oracle.unpack(packed0.ctypes.data + s, n, t_o.ctypes.data + pad + shift - lo, 1, to, s,
                           op=op)
        ap = prod.unpack(p_p.data_ptr() + s, n, t_p.data_ptr() + pad + shift - lo, 1, tp, s, op=op)
        assert ao == ap == n
    cuda.cuda.synchronize()
    used = red_launches(prod) - before
    assert_same_bytes(host_of(cuda, t_p), t_o, f"{ctor} op {op}")
    prod.type_free(tp)
    oracle.type_free(to)
    return used


def overlapping_offsets(rng, nblk, span, sort):
    offs = rng.integers(0, span, nblk)
    return (np.sort(offs) if sort else offs).tolist()


@pytest.mark.parametrize("name,h,es", INT_TYPES)
@pytest.mark.parametrize("op", RED_OPS)
@pytest.mark.parametrize("sort", [True, False])
def test_red_indexed_block(cuda, prod, oracle, name, h, es, op, sort):
    """2^14 blocks of 8 elements over 4096 elements: every element is hit about 32
    times."""
    rng = np.random.default_rng(op * 7 + es + sort)
    offs = overlapping_offsets(rng, 1 << 14, 4096, sort)
    used = unpack_case(cuda, prod, oracle, "type_create_indexed_block", (8, offs), h, es, op,
                       seed=op + 100 * es)
    assert used == 1


@pytest.mark.parametrize("bl", [1, 3, 5, 12])
@pytest.mark.parametrize("op", [yk.OP_SUM, yk.OP_MAX, yk.OP_BXOR])
def test_red_block_lengths(cuda, prod, oracle, bl, op):
    """Block lengths that are not powers of two, hindexed_block byte offsets (elements
    of 8 bytes at multiples of 8) in random order."""
    rng = np.random.default_rng(bl * 31 + op)
    offs = (rng.integers(0, 3000, 5000) * 8).tolist()
    used = unpack_case(cuda, prod, oracle, "type_create_hindexed_block", (bl, offs),
                       yk.TYPE_INT64_T, 8, op, seed=bl)
    assert used == 1


@pytest.mark.parametrize("op", [yk.OP_SUM, yk.OP_MAX, yk.OP_BXOR])
@pytest.mark.parametrize("where", ["fits", "offset_over", "table_over", "negative"])
def test_red_offsets_at_32_bits(cuda, prod, oracle, op, where):
    """Overlapping int32 blocks of 8 (32 bytes) at byte displacements around 2^31 in
    random order: every target offset in 32 bits (the form with a shift and 32-bit
    offsets); a table that fits in 32 bits with one block reaching past 2^31 - 1 (the
    32-bit table with 64-bit offsets); one displacement of 2^31 (the 64-bit table); and
    displacements from -2^31 up.  The typed buffer spans only the blocks: its pointer is
    offset by the lowest displacement."""
    rng = np.random.default_rng(op * 13 + len(where))
    start = -(1 << 31) if where == "negative" else (1 << 31) - 64 - 4096
    offs = (start + rng.integers(0, 1024, 3000) * 4).tolist()
    if where == "offset_over":
        offs.append((1 << 31) - 16)     # its last element ends at 2^31 + 15
    elif where == "table_over":
        offs.append(1 << 31)
    rng.shuffle(offs)
    used = unpack_case(cuda, prod, oracle, "type_create_hindexed_block", (8, offs),
                       yk.TYPE_INT32_T, 4, op, seed=op)
    assert used == 1


@pytest.mark.parametrize("op", [yk.OP_SUM, yk.OP_MIN, yk.OP_BOR])
def test_red_segments(cuda, prod, oracle, op):
    """The packed range cut into 9 segments at element (not block) boundaries: each
    segment is its own launch over part of the blocks."""
    rng = np.random.default_rng(op)
    offs = overlapping_offsets(rng, 6000, 20000, True)
    used = unpack_case(cuda, prod, oracle, "type_create_indexed_block", (6, offs),
                       yk.TYPE_INT32_T, 4, op, seed=op, nseg=9)
    assert used >= 2


@pytest.mark.parametrize("op", [yk.OP_SUM, yk.OP_MAX, yk.OP_BXOR])
def test_red_equal_lengths_indexed(cuda, prod, oracle, op):
    """indexed with equal block lengths: the same overlapping shape."""
    rng = np.random.default_rng(op + 5)
    offs = overlapping_offsets(rng, 4000, 3000, False)
    used = unpack_case(cuda, prod, oracle, "type_create_indexed", ([4] * 4000, offs),
                       yk.TYPE_INT32_T, 4, op, seed=op)
    assert used == 1


@pytest.mark.parametrize("op", [yk.OP_SUM, yk.OP_MIN, yk.OP_BAND])
@pytest.mark.parametrize("name,h,es", [("int32", yk.TYPE_INT32_T, 4), ("int64", yk.TYPE_INT64_T, 8)])
def test_red_overlapping_vector(cuda, prod, oracle, op, name, h, es):
    """hvector of 7-element blocks at a stride of 3 elements: one VEC level whose blocks
    overlap their neighbours."""
    used = unpack_case(cuda, prod, oracle, "type_create_hvector", (5000, 7, 3 * es), h, es, op,
                       seed=op + es, nseg=3)
    assert used >= 1


@pytest.mark.parametrize("ctor_h,es,op,shift", [
    (yk.TYPE_INT32_T, 4, yk.OP_PROD, 0),         # PROD: the ordered kernels
    (yk.TYPE_INT32_T, 4, yk.OP_LAND, 0),
    (yk.TYPE_INT16_T, 2, yk.OP_SUM, 0),          # 2-byte integers
    (yk.TYPE_DOUBLE, 8, yk.OP_MAX, 0),           # floating point (values in [-1, 1))
    (yk.TYPE_INT32_T, 4, yk.OP_SUM, 2),          # typed buffer off the element size
    (yk.TYPE_INT64_T, 8, yk.OP_BXOR, 4),
])
def test_red_not_applied(cuda, prod, oracle, ctor_h, es, op, shift):
    rng = np.random.default_rng(es + op + shift)
    offs = overlapping_offsets(rng, 3000, 2000, True)
    used = unpack_case(cuda, prod, oracle, "type_create_indexed_block", (8, offs), ctor_h, es, op,
                       seed=op, shift=shift, base="double" if ctor_h == yk.TYPE_DOUBLE else "int32")
    assert used == 0


@pytest.mark.parametrize("op", RED_OPS)
def test_red_switched_off_gives_the_same_bytes(cuda, prod, oracle, op):
    """With the form off, the owner kernels run on the same sorted case; both match the
    oracle, and the form is back on afterwards."""
    rng = np.random.default_rng(op + 77)
    offs = overlapping_offsets(rng, 1 << 13, 3000, True)
    red_launches(prod, 0)
    try:
        used = unpack_case(cuda, prod, oracle, "type_create_indexed_block", (8, offs),
                           yk.TYPE_INT64_T, 8, op, seed=op)
        assert used == 0
    finally:
        red_launches(prod, 1)
    assert unpack_case(cuda, prod, oracle, "type_create_indexed_block", (8, offs),
                       yk.TYPE_INT64_T, 8, op, seed=op) == 1


def test_red_extreme_values(cuda, prod, oracle):
    """Sums that wrap, and MAX/MIN over INT_MIN/INT_MAX and -1 (all ones), on blocks
    that all land on the same 8 elements (offsets all 0: one VEC level of stride 0)."""
    for name, h, es, dt in (("int32", yk.TYPE_INT32_T, 4, np.int32),
                            ("int64", yk.TYPE_INT64_T, 8, np.int64)):
        info = np.iinfo(dt)
        vals = np.array([info.min, info.max, -1, 0, 1, info.min + 1, info.max - 1], dtype=dt)
        for op in RED_OPS:
            nblk = 700
            tp = prod.type_create_indexed_block(8, [0] * nblk, h)
            to = oracle.type_create_indexed_block(8, [0] * nblk, h)
            rng = np.random.default_rng(op)
            packed = vals[rng.integers(0, len(vals), nblk * 8)].view(np.uint8).copy()
            typed = vals[rng.integers(0, len(vals), 8)].view(np.uint8).copy()
            t_o = typed.copy()
            t_p, p_p = dev_copy(cuda, typed), dev_copy(cuda, packed)
            before = red_launches(prod)
            oracle.unpack(packed.ctypes.data, packed.nbytes, t_o.ctypes.data, 1, to, 0, op=op)
            prod.unpack(p_p.data_ptr(), packed.nbytes, t_p.data_ptr(), 1, tp, 0, op=op)
            cuda.cuda.synchronize()
            assert red_launches(prod) - before == 1
            assert_same_bytes(host_of(cuda, t_p), t_o, f"{name} op {op}")
            prod.type_free(tp)
            oracle.type_free(to)


def test_red_through_server(cuda, prod, oracle):
    """The persistent server's reduction items: requests of about 0.5-1 MB, cut into many
    items that run on different CTAs in any order, each against the oracle; the server
    is destroyed before the library is used again."""
    srv = yk.Server(prod)
    try:
        cases = [(yk.TYPE_INT64_T, 8, yk.OP_MAX, True), (yk.TYPE_UINT32_T, 4, yk.OP_BXOR, True),
                 (yk.TYPE_INT32_T, 4, yk.OP_SUM, False), (yk.TYPE_INT64_T, 8, yk.OP_BAND, False)]
        for k, (h, es, op, sort) in enumerate(cases):
            rng = np.random.default_rng(900 + k)
            offs = overlapping_offsets(rng, 1 << 14, 20000, sort)
            tp = prod.type_create_indexed_block(8, offs, h)
            to = oracle.type_create_indexed_block(8, offs, h)
            lo, text = oracle.true_extent(to)
            P = oracle.size(to)
            typed0 = fill(rng, text, "int32")
            packed0 = fill(rng, P, "int32")
            t_o = typed0.copy()
            oracle.unpack(packed0.ctypes.data, P, t_o.ctypes.data - lo, 1, to, 0, op=op)
            t_p, p_p = dev_copy(cuda, typed0), dev_copy(cuda, packed0)
            o = yk.unpack_op(p_p.data_ptr(), P, t_p.data_ptr() - lo, 1, tp, 0, op=op)
            t = srv.submit(o)
            assert t is not None
            srv.wait(t)
            assert o.actual == P
            assert_same_bytes(host_of(cuda, t_p), t_o, f"server op {op}")
            assert srv.stats()["items"] >= 2
            prod.type_free(tp)
            oracle.type_free(to)
    finally:
        srv.destroy()


@pytest.mark.parametrize("op", [yk.OP_SUM, yk.OP_BXOR])
def test_red_not_sent_to_host_memory(cuda, prod, oracle, op):
    """A typed buffer in pinned host memory, which the GPU addresses in place over the
    C2C link: the reductions stay on device memory, so the owner kernels run, and the
    bytes match the oracle."""
    rng = np.random.default_rng(op + 300)
    offs = overlapping_offsets(rng, 3000, 2000, True)
    tp = prod.type_create_indexed_block(8, offs, yk.TYPE_INT32_T)
    to = oracle.type_create_indexed_block(8, offs, yk.TYPE_INT32_T)
    lo, text = oracle.true_extent(to)
    P = oracle.size(to)
    typed0 = fill(rng, text, "int32")
    packed0 = fill(rng, P, "int32")
    t_o = typed0.copy()
    oracle.unpack(packed0.ctypes.data, P, t_o.ctypes.data - lo, 1, to, 0, op=op)
    t_h = cuda.from_numpy(typed0.copy()).pin_memory()
    p_p = dev_copy(cuda, packed0)
    before = red_launches(prod)
    prod.unpack(p_p.data_ptr(), P, t_h.data_ptr() - lo, 1, tp, 0, op=op)
    cuda.cuda.synchronize()
    assert red_launches(prod) - before == 0
    assert_same_bytes(t_h.numpy(), t_o, f"host target op {op}")
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("op", [yk.OP_SUM, yk.OP_MAX, yk.OP_BXOR])
def test_red_overlapping_elements(cuda, prod, oracle, op):
    """count > 1 elements whose extent is shorter than their span (8 int64 each, extent
    32 bytes): the overlap comes from the element level of the launch, which the
    reduction form takes as one VEC level over a run."""
    cp, co = prod.type_create_contig(8, yk.TYPE_INT64_T), oracle.type_create_contig(8, yk.TYPE_INT64_T)
    tp, to = prod.type_create_resized(cp, 0, 32), oracle.type_create_resized(co, 0, 32)
    count = 5000
    rng = np.random.default_rng(op + 11)
    typed0 = fill(rng, 32 * (count - 1) + 64, "int64")
    packed0 = fill(rng, 64 * count, "int64")
    t_o = typed0.copy()
    oracle.unpack(packed0.ctypes.data, packed0.nbytes, t_o.ctypes.data, count, to, 0, op=op)
    t_p, p_p = dev_copy(cuda, typed0), dev_copy(cuda, packed0)
    before = red_launches(prod)
    prod.unpack(p_p.data_ptr(), packed0.nbytes, t_p.data_ptr(), count, tp, 0, op=op)
    cuda.cuda.synchronize()
    assert red_launches(prod) - before == 1
    assert_same_bytes(host_of(cuda, t_p), t_o, f"overlapping elements op {op}")
    for y, t in ((prod, tp), (prod, cp), (oracle, to), (oracle, co)):
        y.type_free(t)
