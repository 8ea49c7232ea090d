"""GPU: the batched request path (yaksa_gb300_*pup_batch*) gives the same bytes as
the oracle, for mixed types, sizes, vector widths and for requests the batch kernel
does not take (operators, overlapping targets, contiguous copies) in the same batch.

Tolerance: byte-identical (REPLACE and integer operators).
"""
import ctypes

import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import Pair, assert_same_bytes, dev_copy, fill, host_of
from typegen import Gen, footprint

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["blocking", "nonblocking", "stream"])
@pytest.mark.parametrize("seed", range(4))
def test_batch_matches_oracle(cuda, prod, oracle, seed, mode):
    rng = np.random.default_rng(seed)
    bases = ["int32", "double", "int8", "float", "int64", "int16"]
    g = Gen(oracle, 9000 + seed, max_depth=3)
    reqs = []
    for i in range(20):
        base = bases[i % len(bases)]
        pair = Pair(prod, oracle, g.gen(base))
        count = int(rng.integers(1, 6))
        lo, hi, size = footprint(oracle, pair.ho, count)
        typed = fill(rng, hi - lo + 64, base)
        packed = fill(rng, size * count + 64, base)
        op = "replace" if i % 5 else ("sum" if base != "int8" else "bxor")
        reqs.append(dict(pair=pair, count=count, lo=lo, size=size, typed=typed, packed=packed,
                         base=base, op=op, kind=i % 2))
    ops = []
    for r in reqs:
        r["t_o"], r["p_o"] = r["typed"].copy(), r["packed"].copy()
        r["t_g"], r["p_g"] = dev_copy(cuda, r["typed"]), dev_copy(cuda, r["packed"])
        n = r["size"] * r["count"]
        tp = r["t_g"].data_ptr() + 32 - r["lo"]
        to = r["t_o"].ctypes.data + 32 - r["lo"]
        opc = yk.OP_NAMES[r["op"]]
        if r["kind"] == 0:
            r["ao"] = oracle.pack(to, r["count"], r["pair"].ho, 0, r["p_o"].ctypes.data, n, op=opc)
            ops.append(yk.pack_op(tp, r["count"], r["pair"].hp, 0, r["p_g"].data_ptr(), n, op=opc))
        else:
            r["ao"] = oracle.unpack(r["p_o"].ctypes.data, n, to, r["count"], r["pair"].ho, 0, op=opc)
            ops.append(yk.unpack_op(r["p_g"].data_ptr(), n, tp, r["count"], r["pair"].hp, 0, op=opc))
    arr = prod.batch_array(ops)
    before = prod.stats()["launches"]
    if mode == "blocking":
        prod.pup_batch(arr)
    elif mode == "nonblocking":
        req = prod.ipup_batch(arr)
        prod.wait(req)
    else:
        s = cuda.cuda.Stream()
        h = ctypes.c_void_p(s.cuda_stream)
        prod.pup_batch_stream(arr, ctypes.addressof(h))
        s.synchronize()
    launches = prod.stats()["launches"] - before
    # the REPLACE requests share launches: far fewer launches than requests
    assert launches < len(ops)
    for r, o in zip(reqs, arr):
        assert o.actual == r["ao"]
        assert_same_bytes(host_of(cuda, r["p_g"]), r["p_o"], f"packed {r['op']}", r["base"])
        assert_same_bytes(host_of(cuda, r["t_g"]), r["t_o"], f"typed {r['op']}", r["base"])
        r["pair"].free()
    g.free()


def test_batch_halo_faces(cuda, prod, oracle):
    """The six depth-2 faces of a 96^3 float grid, packed then unpacked as two batches."""
    n = 96
    specs = [([n, n, 2], [0, 0, 0]), ([n, n, 2], [0, 0, n - 2]), ([n, 2, n], [0, 0, 0]),
             ([n, 2, n], [0, n - 2, 0]), ([2, n, n], [0, 0, 0]), ([2, n, n], [n - 2, 0, 0])]
    tp = [prod.type_create_subarray([n] * 3, s, st, yk.SUBARRAY_ORDER_C, yk.TYPE_FLOAT) for s, st in specs]
    rng = np.random.default_rng(2)
    src = cuda.from_numpy(rng.uniform(-1, 1, n ** 3).astype(np.float32)).cuda()
    dst = cuda.zeros_like(src)
    P = 2 * n * n * 4
    bufs = [cuda.empty(P, dtype=cuda.uint8, device="cuda") for _ in tp]
    arr = prod.batch_array([yk.pack_op(src.data_ptr(), 1, t, 0, b.data_ptr(), P) for t, b in zip(tp, bufs)])
    assert prod.pup_batch(arr) == [P] * 6
    arr = prod.batch_array([yk.unpack_op(b.data_ptr(), P, dst.data_ptr(), 1, t, 0) for t, b in zip(tp, bufs)])
    prod.pup_batch(arr)
    s3, d3 = src.view(n, n, n), dst.view(n, n, n)
    mask = cuda.zeros(n, n, n, dtype=cuda.bool, device="cuda")
    mask[:, :, :2] = mask[:, :, -2:] = mask[:, :2, :] = mask[:, -2:, :] = True
    mask[:2] = mask[-2:] = True
    assert cuda.equal(d3[mask], s3[mask])
    assert int((d3[~mask] != 0).sum()) == 0

    # the same exchange captured once and replayed: the graph binds buffers and types
    dst.zero_()
    g, _ = prod.graph_create([[yk.pack_op(src.data_ptr(), 1, t, 0, b.data_ptr(), P) for t, b in zip(tp, bufs)],
                              [yk.unpack_op(b.data_ptr(), P, dst.data_ptr(), 1, t, 0) for t, b in zip(tp, bufs)]])
    for t in tp:
        prod.type_free(t)       # the graph keeps its own references
    for rep in range(3):
        src.add_(1.0)
        l0 = prod.stats()["launches"]
        prod.graph_launch(g)
        # one batched kernel per direction runs per replay, and is counted as such
        assert prod.stats()["launches"] - l0 == 2
        cuda.cuda.synchronize()
        assert cuda.equal(d3[mask], s3[mask])
    prod.graph_free(g)
