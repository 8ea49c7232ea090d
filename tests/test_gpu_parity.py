"""GPU: bit-exact parity of the GPU engine against the CPU oracle on seeded random
datatypes, every operator each base type defines, partial (segmented) packs, and the
reference's memory kinds (device, pinned host, pageable host).

Tolerance: integer, byte and index results must be byte-identical.  Floating-point
results must be byte-identical too, except that a NaN may differ from the oracle's NaN
in payload/sign (the GPU produces the canonical NaN; the reference's NaN bits depend
on the host CPU).  No test input produces NaN unless the test says so.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import Pair, assert_same_bytes, dev_copy, fill, host_of, roundtrip
from typegen import BASE, VALID_OPS, Gen, footprint

pytestmark = pytest.mark.gpu

REPLACE_BASES = ["int8", "int16", "int32", "int64", "float", "double", "c_complex",
                 "c_double_complex", "short_int", "double_int", "float_int", "bool", "char"]


@pytest.mark.parametrize("seed", range(24))
def test_random_types_replace(cuda, prod, oracle, seed):
    rng = np.random.default_rng(seed)
    base = REPLACE_BASES[seed % len(REPLACE_BASES)]
    g = Gen(oracle, 1000 + seed, max_depth=3)
    for i in range(6):
        r = g.gen(base)
        pair = Pair(prod, oracle, r)
        count = int(rng.integers(1, 5))
        nseg = int(rng.choice([1, 1, 3, 7]))
        pg, po, dg, do, actual = roundtrip(cuda, pair, count, base, "replace", rng, nseg=nseg,
                                           ragged=bool(i % 2))
        for (d, s, ao, ap) in actual:
            assert ao == ap, (d, s, ao, ap, r)
        assert_same_bytes(pg, po, f"packed {r}")
        assert_same_bytes(dg, do, f"unpacked {r}")
        pair.free()
    g.free()


OP_BASES = ["int8", "int16", "int32", "int64", "uint32", "float", "double", "c_complex",
            "c_double_complex", "bool", "2int"]


@pytest.mark.parametrize("seed", range(33))
def test_random_types_ops(cuda, prod, oracle, seed):
    rng = np.random.default_rng(seed)
    base = OP_BASES[seed % len(OP_BASES)]
    g = Gen(oracle, 2000 + seed, max_depth=2)
    ops = VALID_OPS[base]
    for i in range(len(ops)):
        op = ops[i]
        r = g.gen(base)
        pair = Pair(prod, oracle, r)
        count = int(rng.integers(1, 4))
        direction = "pack" if i % 2 else "unpack"
        pg, po, dg, do, actual = roundtrip(cuda, pair, count, base, op, rng,
                                           nseg=int(rng.choice([1, 2, 5])), direction=direction)
        for (d, s, ao, ap) in actual:
            assert ao == ap, (d, s, ao, ap, r, op)
        assert_same_bytes(pg, po, f"packed {op} {r}", base)
        assert_same_bytes(dg, do, f"unpacked {op} {r}", base)
        pair.free()
    g.free()


@pytest.mark.parametrize("seed", range(8))
def test_overlapping_unpack_is_ordered(cuda, prod, oracle, seed):
    """Targets reached more than once are updated in the oracle's sequential order."""
    rng = np.random.default_rng(seed)
    base = ["int32", "double", "int64", "float"][seed % 4]
    g = Gen(oracle, 3000 + seed, max_depth=2, overlap=True)
    for op in ["replace", "sum", "max"]:
        r = g.gen(base)
        pair = Pair(prod, oracle, r)
        pg, po, dg, do, actual = roundtrip(cuda, pair, int(rng.integers(1, 3)), base, op, rng,
                                           direction="unpack")
        assert_same_bytes(dg, do, f"overlap {op} {r}", base)
        pair.free()
    g.free()


def test_sorted_overlapping_blocks_sum(cuda, prod, oracle):
    """indexed_block with sorted, overlapping offsets (the reduction config's shape)."""
    rng = np.random.default_rng(7)
    nblk, bl = 4096, 8
    offs = np.sort(rng.integers(0, nblk * bl - bl, nblk)).astype(np.int64)
    for base, op in (("double", "sum"), ("int64", "max"), ("uint32", "bxor"),
                     ("c_complex", "prod"), ("int32", "replace")):
        h = BASE[base][0]
        tp = prod.type_create_indexed_block_array(nblk, bl, offs.ctypes.data, h)
        to = oracle.type_create_indexed_block_array(nblk, bl, offs.ctypes.data, h)
        es = BASE[base][1]
        packed = fill(rng, nblk * bl * es, base)
        target = fill(rng, nblk * bl * es, base)
        d_o = target.copy()
        oracle.unpack(packed.ctypes.data, packed.nbytes, d_o.ctypes.data, 1, to, 0,
                      op=yk.OP_NAMES[op])
        pk, dv = dev_copy(cuda, packed), dev_copy(cuda, target)
        prod.unpack(pk.data_ptr(), packed.nbytes, dv.data_ptr(), 1, tp, 0, op=yk.OP_NAMES[op])
        assert_same_bytes(host_of(cuda, dv), d_o, f"{base} {op}", base)
        prod.type_free(tp)
        oracle.type_free(to)


@pytest.mark.parametrize("cut", [1, 8, 16])
@pytest.mark.parametrize("bl", [4, 8, 16])
def test_sorted_blocks_segmented(cuda, prod, oracle, bl, cut):
    """Sorted overlapping fixed-length blocks unpacked in several calls whose ranges
    start and end inside blocks: each call keeps the block order within its range.
    cut 8 and 16 put every range boundary on 8 or 16 bytes (the 8- and 16-byte chunk
    kernels of small elements); cut 1 anywhere on an element boundary."""
    rng = np.random.default_rng(100 + bl + cut)
    nblk = 3000
    for base, op in (("int8", "sum"), ("int16", "max"), ("float", "sum"), ("double", "prod"),
                     ("c_double_complex", "sum"), ("int32", "replace"), ("int64", "bxor"),
                     ("uint32", "bxor"), ("float", "min")):
        offs = np.sort(rng.integers(0, nblk * bl // 2, nblk)).astype(np.int64)
        h, es = BASE[base][0], BASE[base][1]
        tp = prod.type_create_indexed_block_array(nblk, bl, offs.ctypes.data, h)
        to = oracle.type_create_indexed_block_array(nblk, bl, offs.ctypes.data, h)
        total = nblk * bl * es
        packed = fill(rng, total, base)
        target = fill(rng, (nblk * bl // 2 + bl) * es, base)
        d_o = target.copy()
        pk, dv = dev_copy(cuda, packed), dev_copy(cuda, target)
        g = max(es, cut)
        cuts = sorted(set(int(c) * g for c in rng.integers(1, total // g, 6)))
        bounds = [0] + cuts + [total]
        for s0, s1 in zip(bounds[:-1], bounds[1:]):
            ao = oracle.unpack(packed.ctypes.data + s0, s1 - s0, d_o.ctypes.data, 1, to, s0,
                               op=yk.OP_NAMES[op])
            ap = prod.unpack(pk.data_ptr() + s0, s1 - s0, dv.data_ptr(), 1, tp, s0, op=yk.OP_NAMES[op])
            assert ao == ap
        assert_same_bytes(host_of(cuda, dv), d_o, f"bl {bl} {base} {op}", base)
        prod.type_free(tp)
        oracle.type_free(to)


@pytest.mark.parametrize("bl", [8, 256, 2048, 4096])
def test_sorted_blocks_clustered(cuda, prod, oracle, bl):
    """Sorted blocks of 64 B to 32 KiB where runs of up to 60 blocks share one offset, so
    that one target element folds in contributions from up to 60 blocks, in block order,
    and ranges that start and end inside blocks."""
    rng = np.random.default_rng(300 + bl)
    nblk = max(64, (1 << 21) // (bl * 8))
    span = nblk * bl // 2
    offs = np.sort(rng.integers(0, span, nblk)).astype(np.int64)
    i = 0
    while i < nblk:                     # clusters of equal offsets
        k = int(rng.integers(1, 61))
        offs[i:i + k] = offs[i]
        i += k + int(rng.integers(0, 40))
    for base, op in (("double", "sum"), ("int32", "bxor")):
        h, es = BASE[base][0], BASE[base][1]
        n = bl * 8 // es                # the same block bytes for either base
        eoffs = offs * 8 // es          # kept alive while the constructors read it
        tp = prod.type_create_indexed_block_array(nblk, n, eoffs.ctypes.data, h)
        to = oracle.type_create_indexed_block_array(nblk, n, eoffs.ctypes.data, h)
        total = nblk * bl * 8
        packed = fill(rng, total, base)
        target = fill(rng, (span + bl) * 8, base)
        d_o = target.copy()
        pk, dv = dev_copy(cuda, packed), dev_copy(cuda, target)
        cuts = sorted(set(int(c) * 8 for c in rng.integers(1, total // 8, 4)))
        bounds = [0] + cuts + [total]
        for s0, s1 in zip(bounds[:-1], bounds[1:]):
            ao = oracle.unpack(packed.ctypes.data + s0, s1 - s0, d_o.ctypes.data, 1, to, s0,
                               op=yk.OP_NAMES[op])
            ap = prod.unpack(pk.data_ptr() + s0, s1 - s0, dv.data_ptr(), 1, tp, s0, op=yk.OP_NAMES[op])
            assert ao == ap
        assert_same_bytes(host_of(cuda, dv), d_o, f"bl {bl} {base} {op}", base)
        prod.type_free(tp)
        oracle.type_free(to)


DENSE_STRUCTS = [
    # (blocklengths, displacements, types, resized extent or None)
    ([1, 3], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT], 32),        # 20 B run in 32 B
    ([1, 1], [0, 12], [yk.TYPE_INT64_T, yk.TYPE_FLOAT], 24),       # two segments with a gap
    ([3, 1, 2], [0, 6, 12], [yk.TYPE_INT16_T, yk.TYPE_INT8_T, yk.TYPE_INT16_T], 16),
    ([5], [4], [yk.TYPE_INT32_T], 28),                             # run starting at 4
    ([1, 2], [0, 8], [yk.TYPE_DOUBLE, yk.TYPE_FLOAT], None),       # natural extent 16
    ([7], [0], [yk.TYPE_INT8_T], 12),                              # 1-byte units
    ([60, 1], [0, 248], [yk.TYPE_INT32_T, yk.TYPE_INT32_T], 256),  # 244 B over 256 B
    ([4, 1], [0, 32], [yk.TYPE_INT64_T, yk.TYPE_INT32_T], 48),     # 36 B run in 48 B
    ([3], [0], [yk.TYPE_DOUBLE], 32),                              # 24 B run, 8-byte units
]


@pytest.mark.parametrize("k", range(len(DENSE_STRUCTS)))
def test_dense_struct_pack(cuda, prod, oracle, k):
    """Packs of many elements of dense structs (runs of 7 to 244 bytes in extents of 12
    to 256, one or several segments, 1- to 4-byte units): whole and partial ranges on
    builtin boundaries, packed pointers on and off 16 bytes."""
    bl, dp, ty, ext = DENSE_STRUCTS[k]
    rng = np.random.default_rng(500 + k)

    def mk(y):
        t = y.type_create_struct(bl, dp, ty)
        if ext is None:
            return t
        r = y.type_create_resized(t, 0, ext)
        y.type_free(t)
        return r
    tp, to = mk(prod), mk(oracle)
    size = prod.size(tp)
    for count in (2, 7, 411, 5000):
        lo, hi, _ = footprint(oracle, to, count)
        total = size * count
        typed = fill(rng, hi - lo + 64, "int8")
        tg = dev_copy(cuda, typed)
        cases = [(0, total), (size, total - 2 * size), (0, total // 3)]
        for shift in (0, 4):
            for off, n in cases:
                exp = np.zeros(total + 64, dtype=np.uint8)
                a = oracle.pack(typed.ctypes.data + 32 - lo, count, to, off, exp.ctypes.data, n)
                pk = cuda.zeros(total + 64, dtype=cuda.uint8, device="cuda")
                got = prod.pack(tg.data_ptr() + 32 - lo, count, tp, off, pk.data_ptr() + shift, n)
                assert got == a
                assert np.array_equal(host_of(cuda, pk)[shift:shift + a], exp[:a]), (count, off, n, shift)
    prod.type_free(tp)
    oracle.type_free(to)


def test_dense_struct_pack_byte_kernels(cuda):
    """The dense-struct packs again in a child process with YAKSA_GB300_RUNS_PACK=0, so
    the byte kernels take the struct-like runs too."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-p", "no:cacheprovider",
                        os.path.join(here, "test_gpu_parity.py"), "-k",
                        "dense_struct_pack and not byte_kernels"],
                       env=dict(os.environ, YAKSA_GB300_RUNS_PACK="0"),
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]


def test_nonblocking_and_stream(cuda, prod, oracle):
    t = prod.type_create_hvector(1024, 4, 128, yk.TYPE_DOUBLE)
    src = cuda.randn(1024 * 16, dtype=cuda.float64, device="cuda")
    out = cuda.zeros(1024 * 4, dtype=cuda.float64, device="cuda")
    n, req = prod.ipack(src.data_ptr(), 1, t, 0, out.data_ptr(), out.numel() * 8)
    assert n == 32768
    while not prod.test(req):
        pass
    ref = src.view(1024, 16)[:, :4].reshape(-1)
    assert cuda.equal(out, ref)
    back = cuda.zeros_like(src)
    n, req = prod.iunpack(out.data_ptr(), 32768, back.data_ptr(), 1, t, 0)
    prod.wait(req)
    assert cuda.equal(back.view(1024, 16)[:, :4], src.view(1024, 16)[:, :4])
    # stream-ordered: enqueue on a user stream, synchronize it
    import ctypes
    s = cuda.cuda.Stream()
    handle = ctypes.c_void_p(s.cuda_stream)
    out2 = cuda.zeros_like(out)
    prod.pack_stream(src.data_ptr(), 1, t, 0, out2.data_ptr(), 32768, ctypes.addressof(handle))
    s.synchronize()
    assert cuda.equal(out2, ref)
    prod.type_free(t)


@pytest.mark.parametrize("kind", ["pinned", "pageable"])
def test_host_buffers(cuda, prod, oracle, kind):
    """Host buffers: served in place over the C2C link or staged; same bytes either way."""
    rng = np.random.default_rng(11)
    sizes, subs, starts = [64, 64, 64], [64, 64, 2], [0, 0, 62]
    tp = prod.type_create_subarray(sizes, subs, starts, yk.SUBARRAY_ORDER_C, yk.TYPE_FLOAT)
    to = oracle.type_create_subarray(sizes, subs, starts, yk.SUBARRAY_ORDER_C, yk.TYPE_FLOAT)
    grid = rng.uniform(-1, 1, 64 ** 3).astype(np.float32)
    if kind == "pinned":
        hg = cuda.from_numpy(grid).pin_memory()
        hp = cuda.zeros(64 * 64 * 2, dtype=cuda.float32).pin_memory()
        gptr, pptr = hg.data_ptr(), hp.data_ptr()
        get = lambda: hp.numpy()
    else:
        hg_np = grid.copy()
        hp_np = np.zeros(64 * 64 * 2, dtype=np.float32)
        gptr, pptr = hg_np.ctypes.data, hp_np.ctypes.data
        get = lambda: hp_np
    ref = np.zeros(64 * 64 * 2, dtype=np.float32)
    oracle.pack(grid.ctypes.data, 1, to, 0, ref.ctypes.data, ref.nbytes)
    n = prod.pack(gptr, 1, tp, 0, pptr, ref.nbytes)
    assert n == ref.nbytes
    assert np.array_equal(get(), ref)
    prod.type_free(tp)
    oracle.type_free(to)
