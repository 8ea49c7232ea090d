"""GPU: yaksa_gb300_pup_noalloc (descriptor tables in a static device array instead of
a per-type allocation) gives the same bytes as yaksa_pack_stream/yaksa_unpack_stream,
on two calls in a row, for table-driven types (hindexed, struct segments, sorted
overlapping blocks under operators), table-free types and contiguous types; requests
whose tables exceed the array are refused before anything runs.

This file is collected last so that it also runs after every other GPU test in one
process; it passes alone as well.

Tolerance: byte-identical (the two entry points run the same kernels on the same
inputs; no input here produces NaN).
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


def _run(cuda, prod, t, count, kind, op, typed0, packed0, lo, path):
    """One request from fresh buffers; returns (typed, packed, actual) after it."""
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


def _bounds(prod, t, count):
    lb, text = prod.true_extent(t)
    ext = prod.extent(t)[1]
    return min(lb, lb + (count - 1) * ext), max(lb + text, lb + text + (count - 1) * ext)


def _same_as_plain(cuda, prod, t, count, base, op=yk.OP_REPLACE, seed=0, bounds=None):
    rng = np.random.default_rng(seed)
    lo, hi = bounds if bounds else _bounds(prod, t, count)
    typed0 = fill(rng, hi - lo, base)
    packed0 = fill(rng, prod.size(t) * count, base)
    for kind in ((1,) if op != yk.OP_REPLACE else (0, 1)):
        ref = _run(cuda, prod, t, count, kind, op, typed0, packed0, lo, "plain")
        for call in range(2):
            got = _run(cuda, prod, t, count, kind, op, typed0, packed0, lo, "noalloc")
            assert got[2] == ref[2], (kind, call)
            assert np.array_equal(got[0], ref[0]), (kind, call, "typed")
            assert np.array_equal(got[1], ref[1]), (kind, call, "packed")


def test_noalloc_hindexed(cuda, prod):
    rng = np.random.default_rng(1)
    nb = 3000
    blens = rng.integers(1, 40, nb)
    displs = (np.cumsum(blens + rng.integers(0, 9, nb)) - blens) * 4
    perm = rng.permutation(nb)
    t = prod.type_create_hindexed(blens[perm].tolist(), displs[perm].tolist(), yk.TYPE_INT32_T)
    _same_as_plain(cuda, prod, t, 2, "int32")
    prod.type_free(t)


def test_noalloc_struct_segments(cuda, prod):
    t = prod.type_create_struct([1, 2, 3], [0, 12, 24], [yk.TYPE_INT32_T, yk.TYPE_DOUBLE, yk.TYPE_INT16_T])
    _same_as_plain(cuda, prod, t, 5, "int8")
    prod.type_free(t)


@pytest.mark.parametrize("base,h,op", [("double", yk.TYPE_DOUBLE, yk.OP_SUM),
                                       ("int64", yk.TYPE_INT64_T, yk.OP_MAX),
                                       ("int32", yk.TYPE_INT32_T, yk.OP_REPLACE)])
def test_noalloc_overlapping_blocks(cuda, prod, base, h, op):
    rng = np.random.default_rng(2)
    offs = np.sort(rng.integers(0, 5000, 1500)).tolist()
    t = prod.type_create_indexed_block(8, offs, h)
    _same_as_plain(cuda, prod, t, 1, base, op=op)
    prod.type_free(t)


def test_noalloc_table_free_and_contiguous(cuda, prod):
    v = prod.type_create_hvector(300, 3, 40, yk.TYPE_FLOAT)
    _same_as_plain(cuda, prod, v, 3, "float")
    c = prod.type_create_contig(1000, yk.TYPE_INT64_T)
    _same_as_plain(cuda, prod, c, 2, "int64")
    prod.type_free(v)
    prod.type_free(c)


@pytest.mark.parametrize("seed", range(4))
def test_noalloc_random_types(cuda, prod, oracle, seed):
    g = Gen(oracle, 7000 + seed, max_depth=3)
    for i, base in enumerate(["int32", "double", "int8", "float"]):
        pair = Pair(prod, oracle, g.gen(base))
        count = 1 + i % 3
        lo, hi, _ = footprint(oracle, pair.ho, count)
        _same_as_plain(cuda, prod, pair.hp, count, base, seed=seed, bounds=(lo, hi))
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
