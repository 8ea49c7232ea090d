"""GPU: yaksa_gb300_pup_noalloc, the pack/unpack entry point for callers that cannot
allocate device memory (a library whose device memory is all owned by the application's
allocator, or code issuing requests beside a resident persistent kernel, where a cudaFree
would synchronize the device).  Its descriptor tables travel with each request into a
static device array instead of a per-type allocation.

Each case runs the entry point twice in a row and compares both results byte for byte
with the oracle and with yaksa_pack_stream/yaksa_unpack_stream on the same inputs:
table-driven types (hindexed, struct segments, sorted overlapping blocks under operators),
table-free types and contiguous types.  Requests whose tables exceed the array, and
records whose kind is neither pack nor unpack, are refused before anything runs.  With
the library's next device allocation armed to fail, the entry point still succeeds on a
type that was never packed (it allocated nothing), while the plain path then fails.

This file is collected last so that it also runs after every other GPU test in one
process; it passes alone as well.

Tolerance: byte-identical (no input here produces NaN).
"""
import ctypes

import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import Pair, fill
from typegen import Gen, footprint

pytestmark = pytest.mark.gpu


def _stream(cuda):
    h = ctypes.c_void_p(cuda.cuda.current_stream().cuda_stream)
    return h, ctypes.addressof(h)


def _both(prod, oracle, ctor, *args):
    """The same constructor call on the product and on the oracle."""
    return getattr(prod, ctor)(*args), getattr(oracle, ctor)(*args)


def _run(cuda, prod, t, count, kind, op, typed0, packed0, lo, path):
    """One request from fresh device buffers; returns (typed, packed, actual) after it."""
    tg = cuda.from_numpy(typed0.copy()).cuda()
    pg = cuda.from_numpy(packed0.copy()).cuda()
    cuda.cuda.synchronize()
    h, sp = _stream(cuda)
    n = len(packed0)
    tp = tg.data_ptr() - lo
    if path == "plain":
        if kind == 0:
            actual = prod.pack_stream(tp, count, t, 0, pg.data_ptr(), n, sp, op=op)
        else:
            actual = prod.unpack_stream(pg.data_ptr(), n, tp, count, t, 0, sp, op=op)
    else:
        o = (yk.pack_op(tp, count, t, 0, pg.data_ptr(), n, op=op) if kind == 0 else
             yk.unpack_op(pg.data_ptr(), n, tp, count, t, 0, op=op))
        assert prod.pup_noalloc(o, sp) == yk.SUCCESS
        actual = o.actual
    cuda.cuda.synchronize()
    return tg.cpu().numpy(), pg.cpu().numpy(), actual


def _run_oracle(oracle, t, count, kind, op, typed0, packed0, lo):
    th, ph = typed0.copy(), packed0.copy()
    n = len(ph)
    if kind == 0:
        actual = oracle.pack(th.ctypes.data - lo, count, t, 0, ph.ctypes.data, n, op=op)
    else:
        actual = oracle.unpack(ph.ctypes.data, n, th.ctypes.data - lo, count, t, 0, op=op)
    return th, ph, actual


def _bounds(prod, t, count):
    lb, text = prod.true_extent(t)
    ext = prod.extent(t)[1]
    return min(lb, lb + (count - 1) * ext), max(lb + text, lb + text + (count - 1) * ext)


def _check(cuda, prod, oracle, tp, to, count, base, op=yk.OP_REPLACE, seed=0, bounds=None):
    rng = np.random.default_rng(seed)
    lo, hi = bounds if bounds else _bounds(prod, tp, count)
    typed0 = fill(rng, hi - lo, base)
    packed0 = fill(rng, prod.size(tp) * count, base)
    for kind in ((1,) if op != yk.OP_REPLACE else (0, 1)):
        exp = _run_oracle(oracle, to, count, kind, op, typed0, packed0, lo)
        ref = _run(cuda, prod, tp, count, kind, op, typed0, packed0, lo, "plain")
        for call in range(2):
            got = _run(cuda, prod, tp, count, kind, op, typed0, packed0, lo, "noalloc")
            for name, want in (("oracle", exp), ("plain", ref)):
                assert got[2] == want[2], (kind, call, name)
                assert np.array_equal(got[0], want[0]), (kind, call, name, "typed")
                assert np.array_equal(got[1], want[1]), (kind, call, name, "packed")


def _hindexed_arrays(rng, nb, esize, gap=9):
    blens = rng.integers(1, 40, nb)
    displs = (np.cumsum(blens + rng.integers(0, gap, nb)) - blens) * esize
    perm = rng.permutation(nb)
    return blens[perm].tolist(), displs[perm].tolist()


def test_noalloc_hindexed(cuda, prod, oracle):
    bl, ds = _hindexed_arrays(np.random.default_rng(1), 3000, 4)
    tp, to = _both(prod, oracle, "type_create_hindexed", bl, ds, yk.TYPE_INT32_T)
    _check(cuda, prod, oracle, tp, to, 2, "int32")
    prod.type_free(tp)
    oracle.type_free(to)


def test_noalloc_struct_segments(cuda, prod, oracle):
    tp, to = _both(prod, oracle, "type_create_struct", [1, 2, 3], [0, 12, 24],
                   [yk.TYPE_INT32_T, yk.TYPE_DOUBLE, yk.TYPE_INT16_T])
    _check(cuda, prod, oracle, tp, to, 5, "int8")
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("base,h,op", [("double", yk.TYPE_DOUBLE, yk.OP_SUM),
                                       ("int64", yk.TYPE_INT64_T, yk.OP_MAX),
                                       ("int32", yk.TYPE_INT32_T, yk.OP_REPLACE)])
def test_noalloc_overlapping_blocks(cuda, prod, oracle, base, h, op):
    rng = np.random.default_rng(2)
    offs = np.sort(rng.integers(0, 5000, 1500)).tolist()
    tp, to = _both(prod, oracle, "type_create_indexed_block", 8, offs, h)
    _check(cuda, prod, oracle, tp, to, 1, base, op=op)
    prod.type_free(tp)
    oracle.type_free(to)


def test_noalloc_table_free_and_contiguous(cuda, prod, oracle):
    vp, vo = _both(prod, oracle, "type_create_hvector", 300, 3, 40, yk.TYPE_FLOAT)
    _check(cuda, prod, oracle, vp, vo, 3, "float")
    cp, co = _both(prod, oracle, "type_create_contig", 1000, yk.TYPE_INT64_T)
    _check(cuda, prod, oracle, cp, co, 2, "int64")
    for y, t in ((prod, vp), (prod, cp), (oracle, vo), (oracle, co)):
        y.type_free(t)


@pytest.mark.parametrize("seed", range(4))
def test_noalloc_random_types(cuda, prod, oracle, seed):
    g = Gen(oracle, 7000 + seed, max_depth=3)
    for i, base in enumerate(["int32", "double", "int8", "float"]):
        pair = Pair(prod, oracle, g.gen(base))
        count = 1 + i % 3
        lo, hi, _ = footprint(oracle, pair.ho, count)
        _check(cuda, prod, oracle, pair.hp, pair.ho, count, base, seed=seed, bounds=(lo, hi))
        pair.free()
    g.free()


def test_noalloc_back_to_back_types(cuda, prod):
    """Two requests of different table-driven types enqueued back to back on one stream:
    the second request's tables overwrite the first's only after the first kernel."""
    rng = np.random.default_rng(3)
    types, bufs = [], []
    for k in range(2):
        nb = 2000 + 1000 * k
        blens = rng.integers(1, 30, nb)
        displs = (np.cumsum(blens + rng.integers(0, 5, nb)) - blens) * 8
        t = prod.type_create_hindexed(blens[rng.permutation(nb)].tolist(),
                                      displs[rng.permutation(nb)].tolist(), yk.TYPE_DOUBLE)
        typed = cuda.from_numpy(fill(rng, _bounds(prod, t, 1)[1], "double")).cuda()
        out_plain = cuda.zeros(prod.size(t), dtype=cuda.uint8, device="cuda")
        out_na = cuda.zeros(prod.size(t), dtype=cuda.uint8, device="cuda")
        types.append(t)
        bufs.append((typed, out_plain, out_na))
    cuda.cuda.synchronize()
    h, sp = _stream(cuda)
    for t, (typed, op_, _) in zip(types, bufs):
        prod.pack_stream(typed.data_ptr(), 1, t, 0, op_.data_ptr(), op_.numel(), sp)
    ops = [yk.pack_op(typed.data_ptr(), 1, t, 0, na.data_ptr(), na.numel())
           for t, (typed, _, na) in zip(types, bufs)]
    for o in ops:
        assert prod.pup_noalloc(o, sp) == yk.SUCCESS
    cuda.cuda.synchronize()
    for (typed, op_, na) in bufs:
        assert cuda.equal(op_, na)
    for t in types:
        prod.type_free(t)


def test_noalloc_allocates_nothing(cuda, prod, oracle):
    """The library's next device allocation is armed to fail.  The entry point packs and
    unpacks a hindexed type that has never been packed (so it has no device tables yet)
    and succeeds; the armed failure is still pending afterwards, so the plain path's
    first pack of another new table-driven type then reports YAKSA_ERR__OUT_OF_MEM."""
    rng = np.random.default_rng(5)
    bl, ds = _hindexed_arrays(rng, 2500, 4)
    tp, to = _both(prod, oracle, "type_create_hindexed", bl, ds, yk.TYPE_INT32_T)
    bl2, ds2 = _hindexed_arrays(rng, 2600, 4)
    tq = prod.type_create_hindexed(bl2, ds2, yk.TYPE_INT32_T)
    lo, hi = _bounds(prod, tp, 1)
    typed0 = fill(rng, hi - lo, "int32")
    packed0 = fill(rng, prod.size(tp), "int32")
    exp_pack = _run_oracle(oracle, to, 1, 0, yk.OP_REPLACE, typed0, packed0, lo)
    exp_unpack = _run_oracle(oracle, to, 1, 1, yk.OP_REPLACE, typed0, packed0, lo)
    # every device buffer of the test exists before the failure is armed
    tg = cuda.from_numpy(typed0.copy()).cuda()
    pg = cuda.from_numpy(packed0.copy()).cuda()
    pg2 = cuda.from_numpy(packed0.copy()).cuda()
    tg2 = cuda.from_numpy(typed0.copy()).cuda()
    qlo, qhi = _bounds(prod, tq, 1)
    tqd = cuda.zeros(qhi - qlo, dtype=cuda.uint8, device="cuda")
    qout = cuda.zeros(prod.size(tq), dtype=cuda.uint8, device="cuda")
    cuda.cuda.synchronize()
    h, sp = _stream(cuda)
    prod.lib.yaksa_gb300_debug_fail_alloc(1)
    try:
        o = yk.pack_op(tg.data_ptr() - lo, 1, tp, 0, pg.data_ptr(), pg.numel())
        assert prod.pup_noalloc(o, sp) == yk.SUCCESS
        u = yk.unpack_op(pg2.data_ptr(), pg2.numel(), tg2.data_ptr() - lo, 1, tp, 0)
        assert prod.pup_noalloc(u, sp) == yk.SUCCESS
        cuda.cuda.synchronize()
        assert o.actual == exp_pack[2] and u.actual == exp_unpack[2]
        assert np.array_equal(pg.cpu().numpy(), exp_pack[1]), "packed bytes differ from the oracle"
        assert np.array_equal(tg2.cpu().numpy(), exp_unpack[0]), "unpacked bytes differ from the oracle"
        with pytest.raises(yk.YaksaError) as ei:
            prod.pack_stream(tqd.data_ptr() - qlo, 1, tq, 0, qout.data_ptr(), qout.numel(), sp)
        assert ei.value.rc == yk.ERR_OUT_OF_MEM
    finally:
        prod.lib.yaksa_gb300_debug_fail_alloc(0)
    # the failure is not cached: the same plain call now succeeds
    assert prod.pack_stream(tqd.data_ptr() - qlo, 1, tq, 0, qout.data_ptr(), qout.numel(), sp) == \
        prod.size(tq)
    cuda.cuda.synchronize()
    for y, t in ((prod, tp), (prod, tq), (oracle, to)):
        y.type_free(t)


def test_noalloc_rejects_bad_kind(cuda, prod):
    """A record whose kind is neither pack (0) nor unpack (1) is refused; nothing is
    written."""
    t = prod.type_create_hvector(64, 2, 16, yk.TYPE_INT32_T)
    typed = cuda.zeros(64 * 16, dtype=cuda.uint8, device="cuda")
    out = cuda.full((prod.size(t),), 7, dtype=cuda.uint8, device="cuda")
    cuda.cuda.synchronize()
    h, sp = _stream(cuda)
    o = yk.pack_op(typed.data_ptr(), 1, t, 0, out.data_ptr(), out.numel())
    o.kind = 2
    assert prod.pup_noalloc(o, sp) == yk.ERR_INTERNAL
    assert o.actual == 0
    cuda.cuda.synchronize()
    assert int((out != 7).sum()) == 0
    prod.type_free(t)


def test_noalloc_rejects_oversized_tables(cuda, prod):
    """About 600,000 hindexed blocks need more than the 8 MiB array: refused, nothing
    written."""
    rng = np.random.default_rng(4)
    nb = 600_000
    blens = rng.integers(1, 4, nb).astype(np.int64)
    displs = ((np.cumsum(blens + 1) - blens) * 4).astype(np.int64)
    displs = displs[rng.permutation(nb)]
    t = prod.type_create_hindexed_arrays(nb, blens.ctypes.data, displs.ctypes.data, yk.TYPE_INT32_T)
    hi = int(displs.max()) + 16
    typed = cuda.zeros(hi, dtype=cuda.uint8, device="cuda")
    out = cuda.full((prod.size(t),), 7, dtype=cuda.uint8, device="cuda")
    cuda.cuda.synchronize()
    h, sp = _stream(cuda)
    o = yk.pack_op(typed.data_ptr(), 1, t, 0, out.data_ptr(), out.numel())
    assert prod.pup_noalloc(o, sp) == yk.ERR_NOT_SUPPORTED
    assert o.actual == 0
    cuda.cuda.synchronize()
    assert int((out != 7).sum()) == 0
    prod.type_free(t)
