"""GPU: the forms that move data with the tensor memory accelerator, against the oracle:
the TMA (cp.async.bulk.tensor) form of the REPLACE kernels for regular nests, and the
hindexed unpack whose packed stream is staged by cp.async.bulk.

With the test hook set to 2 every launch that has a TMA form takes it: packs of nests of
one to three strided levels over runs of up to 256 bytes (the run may start anywhere in
its 16-byte row; bytes outside it are never read), and unpacks whose runs are whole
16-byte units on 16-byte boundaries (a box store then writes exactly the runs).  The
cases cover partial last boxes, runs at offsets 0, 4 and 8 of a row, 1-, 2- and 3-level
nests, and shapes just outside the rules, which must fall back to the other kernels
with the same bytes.  The TMA launch counter shows which launches took the TMA form, and
no TMA wait may run out.  A last case leaves the choice to the autotuner (hook 1) and
checks that repeated launches of one shape, whichever form runs, give the same bytes.

Tolerance: byte-identical.
"""
import ctypes

import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import dev_copy

pytestmark = pytest.mark.gpu


def _stats(prod):
    n, f = ctypes.c_ulonglong(), ctypes.c_uint()
    assert prod.lib.yaksa_gb300_debug_tma_stats(ctypes.byref(n), ctypes.byref(f)) == 0
    return n.value, f.value


@pytest.fixture
def tma(prod):
    prod.lib.yaksa_gb300_debug_tma.argtypes = [ctypes.c_int]
    prod.lib.yaksa_gb300_debug_tma.restype = ctypes.c_int
    prod.lib.yaksa_gb300_debug_tma_stats.argtypes = [ctypes.POINTER(ctypes.c_ulonglong),
                                                     ctypes.POINTER(ctypes.c_uint)]
    prod.lib.yaksa_gb300_debug_tma_stats.restype = ctypes.c_int
    assert prod.lib.yaksa_gb300_debug_tma(2) == 0
    yield prod
    prod.lib.yaksa_gb300_debug_tma(1)      # the library's default


def _bounds(prod, t, count):
    lb, text = prod.true_extent(t)
    ext = prod.extent(t)[1]
    return min(lb, lb + (count - 1) * ext), max(lb + text, lb + text + (count - 1) * ext)


def _roundtrip(cuda, prod, oracle, tp, to, count, shift=0, seed=0):
    """pack then unpack (into a fresh target) on both libraries; the typed buffer starts
    `shift` bytes past a 256-byte boundary"""
    rng = np.random.default_rng(seed)
    lo, hi = _bounds(prod, tp, count)
    n = prod.size(tp) * count
    typed = rng.integers(0, 256, hi - lo + shift, dtype=np.uint8)
    target = rng.integers(0, 256, hi - lo + shift, dtype=np.uint8)
    # oracle
    ph = np.zeros(n, dtype=np.uint8)
    assert oracle.pack(typed.ctypes.data + shift - lo, count, to, 0, ph.ctypes.data, n) == n
    th = target.copy()
    oracle.unpack(ph.ctypes.data, n, th.ctypes.data + shift - lo, count, to, 0)
    # product
    td, tgt = dev_copy(cuda, typed), dev_copy(cuda, target)
    pd = cuda.zeros(n, dtype=cuda.uint8, device="cuda")
    assert prod.pack(td.data_ptr() + shift - lo, count, tp, 0, pd.data_ptr(), n) == n
    prod.unpack(pd.data_ptr(), n, tgt.data_ptr() + shift - lo, count, tp, 0)
    cuda.cuda.synchronize()
    assert np.array_equal(pd.cpu().numpy(), ph), "packed bytes differ from the oracle"
    assert np.array_equal(tgt.cpu().numpy(), th), "unpacked bytes differ from the oracle"


def _expect(prod, before, packs, unpacks):
    n, f = _stats(prod)
    assert f == 0, "a TMA wait ran out"
    assert n - before == packs + unpacks, (n - before, packs, unpacks)


# (name, constructor, args, count, TMA packs, TMA unpacks per round trip, typed shift)
CASES = [
    ("xface_lo", "type_create_subarray", ([64, 64, 64], [64, 64, 2], [0, 0, 0], 0, 45), 1, 1, 0, 0),
    # the x+ face of an aligned grid starts 248 bytes into each row: 8 bytes into its 16
    ("xface_hi", "type_create_subarray", ([64, 64, 64], [64, 64, 2], [0, 0, 62], 0, 45), 1, 1, 0, 8),
    ("hvector_c0", "type_create_hvector", (1024, 4, 128, 46), 1, 1, 1, 0),
    ("hvector_partial_box", "type_create_hvector", (1000, 4, 48, 45), 1, 1, 1, 0),
    ("hvector_shift4", "type_create_hvector", (777, 3, 64, 45), 1, 1, 0, 4),
    ("subarray_3d_count2", "type_create_subarray", ([40, 30, 24], [10, 7, 12], [3, 5, 4], 0, 45), 2, 1, 1, 0),
    ("run_240", "type_create_hvector", (300, 60, 256, 45), 1, 1, 1, 0),
    ("run_272_falls_back", "type_create_hvector", (100, 68, 288, 45), 1, 0, 0, 0),
    ("stride_not_16_falls_back", "type_create_hvector", (500, 2, 40, 45), 1, 0, 0, 0),
    ("negative_stride_falls_back", "type_create_hvector", (200, 4, -64, 45), 1, 0, 0, 0),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_tma_forced(cuda, tma, oracle, case):
    name, ctor, args, count, npk, nup, shift = case
    prod = tma
    tp, to = getattr(prod, ctor)(*args), getattr(oracle, ctor)(*args)
    before = _stats(prod)[0]
    _roundtrip(cuda, prod, oracle, tp, to, count, shift=shift, seed=len(name))
    _expect(prod, before, npk, nup)
    prod.type_free(tp)
    oracle.type_free(to)


def test_struct_run_pack(cuda, tma, oracle):
    """the 20-byte run of {int64, float x3} in a 32-byte extent: TMA pack, unpack on the
    other kernels (20 bytes are not whole 16-byte units)"""
    prod = tma
    s = [y.type_create_struct([1, 3], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT]) for y in (prod, oracle)]
    tp, to = prod.type_create_resized(s[0], 0, 32), oracle.type_create_resized(s[1], 0, 32)
    before = _stats(prod)[0]
    _roundtrip(cuda, prod, oracle, tp, to, 5000)
    _expect(prod, before, 1, 0)
    for y, t in ((prod, tp), (prod, s[0]), (oracle, to), (oracle, s[1])):
        y.type_free(t)


def test_tma_tuned_repeats(cuda, prod, oracle):
    """hook 1: the autotuner times the TMA form against the other shapes over the first
    launches of a class; every launch's bytes equal the oracle's"""
    prod.lib.yaksa_gb300_debug_tma.argtypes = [ctypes.c_int]
    assert prod.lib.yaksa_gb300_debug_tma(1) == 0
    try:
        n = 256
        args = ([n, n, n], [n, n, 2], [0, 0, n - 2], 0, 45)
        tp, to = prod.type_create_subarray(*args), oracle.type_create_subarray(*args)
        rng = np.random.default_rng(9)
        grid = rng.integers(0, 256, n * n * n * 4, dtype=np.uint8)
        P = prod.size(tp)
        ref = np.zeros(P, dtype=np.uint8)
        oracle.pack(grid.ctypes.data, 1, to, 0, ref.ctypes.data, P)
        gd = dev_copy(cuda, grid)
        outs = [cuda.zeros(P, dtype=cuda.uint8, device="cuda") for _ in range(40)]
        for o in outs:
            prod.pack(gd.data_ptr(), 1, tp, 0, o.data_ptr(), P)
        cuda.cuda.synchronize()
        for o in outs:
            assert np.array_equal(o.cpu().numpy(), ref)
        prod.type_free(tp)
        oracle.type_free(to)
    finally:
        prod.lib.yaksa_gb300_debug_tma(1)


def _bulk_failures(prod):
    f = ctypes.c_uint()
    prod.lib.yaksa_gb300_debug_bulk_failures.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    assert prod.lib.yaksa_gb300_debug_bulk_failures(ctypes.byref(f)) == 0
    return f.value


@pytest.mark.parametrize("maxlen,seed", [(40, 1), (5000, 2)])
def test_hindexed_bulk_unpack(cuda, tma, oracle, maxlen, seed):
    """hook 2 forces the bulk-staged hindexed unpack: shuffled blocks (some longer than
    an 8 KiB tile), a packed size that is not a multiple of 16 (the last tile's tail is
    read with plain loads), the whole request and a part starting on a 16-byte boundary
    in the middle of it"""
    prod = tma
    rng = np.random.default_rng(seed)
    nb = 30001
    blens = rng.integers(1, maxlen, nb)
    blens[0] += (1 - int(blens.sum()) % 2)          # an odd element count: size % 16 != 0
    displs = (np.cumsum(blens + rng.integers(0, 9, nb)) - blens) * 4
    perm = rng.permutation(nb)
    args = (blens[perm].tolist(), displs[perm].tolist(), yk.TYPE_INT32_T)
    tp, to = prod.type_create_hindexed(*args), oracle.type_create_hindexed(*args)
    n = prod.size(tp)
    assert n % 16
    lo, hi = _bounds(prod, tp, 1)
    packed = rng.integers(0, 256, n, dtype=np.uint8)
    target = rng.integers(0, 256, hi - lo, dtype=np.uint8)
    pd = dev_copy(cuda, packed)
    before = _stats(prod)[0]
    for b0, b1 in ((0, n), (16 * (n // 48), n - 4 * 1001)):
        th = target.copy()
        oracle.unpack(packed.ctypes.data + b0, b1 - b0, th.ctypes.data - lo, 1, to, b0)
        td = dev_copy(cuda, target)
        prod.unpack(pd.data_ptr() + b0, b1 - b0, td.data_ptr() - lo, 1, tp, b0)
        cuda.cuda.synchronize()
        assert np.array_equal(td.cpu().numpy(), th), (b0, b1)
    assert _stats(prod)[0] - before == 2, "both unpacks took the bulk-staged form"
    assert _bulk_failures(prod) == 0
    # outside its rules: a packed pointer off 16 bytes, and a pack, take the other kernels
    before = _stats(prod)[0]
    th = target.copy()
    oracle.unpack(packed.ctypes.data + 4, n - 4, th.ctypes.data - lo, 1, to, 4)
    td = dev_copy(cuda, target)
    prod.unpack(pd.data_ptr() + 4, n - 4, td.data_ptr() - lo, 1, tp, 4)
    out = cuda.zeros(n, dtype=cuda.uint8, device="cuda")
    prod.pack(dev_copy(cuda, target).data_ptr() - lo, 1, tp, 0, out.data_ptr(), n)
    cuda.cuda.synchronize()
    assert np.array_equal(td.cpu().numpy(), th)
    ph = np.zeros(n, dtype=np.uint8)
    oracle.pack(target.ctypes.data - lo, 1, to, 0, ph.ctypes.data, n)
    assert np.array_equal(out.cpu().numpy(), ph)
    assert _stats(prod)[0] == before
    prod.type_free(tp)
    oracle.type_free(to)
