"""GPU: the launch-shape autotuner times its candidate shapes on real launches, settles
on one per shape class, and every launch gives the same bytes whichever shape ran
(compared with the first result and with the oracle).

Tolerance: byte-identical (REPLACE).
"""
import ctypes

import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import dev_copy, fill, host_of

pytestmark = pytest.mark.gpu


def test_single_launch_shape_is_tuned_and_exact(cuda, prod, oracle):
    # a 3-level nest with 8-byte runs, 2^18 units: above the tuning threshold
    shapes = []
    for y in (prod, oracle):
        inner = y.type_create_hvector(64, 2, 4096, yk.TYPE_FLOAT)
        t = y.type_create_hvector(64, 1, 64 * 4096 * 2, inner)
        shapes.append((inner, t))
    (pi, pt), (oi, ot) = shapes
    rng = np.random.default_rng(3)
    lo, hi = prod.true_extent(pt)
    n = prod.size(pt) * 8
    ext = prod.extent(pt)[1]
    typed = fill(rng, lo + hi + 7 * ext + 64, "float")
    tg = dev_copy(cuda, typed)
    expect = np.zeros(n, dtype=np.uint8)
    oracle.pack(typed.ctypes.data, 8, ot, 0, expect.ctypes.data, n)
    h = ctypes.c_void_p(cuda.cuda.current_stream().cuda_stream)
    before = prod.autotune_stats()
    for i in range(40):
        out = cuda.zeros(n, dtype=cuda.uint8, device="cuda")
        prod.pack_stream(tg.data_ptr(), 8, pt, 0, out.data_ptr(), n, ctypes.addressof(h))
        cuda.cuda.synchronize()
        assert np.array_equal(host_of(cuda, out), expect), i
    after = prod.autotune_stats()
    assert after["classes"] > before["classes"]
    assert after["decided"] > before["decided"]
    assert after["probes"] >= before["probes"] + 10
    for y, (a, b) in ((prod, shapes[0]), (oracle, shapes[1])):
        y.type_free(b)
        y.type_free(a)


def test_batch_launch_shape_is_tuned_and_exact(cuda, prod, oracle):
    rng = np.random.default_rng(4)
    types = [(prod.type_create_vector(4096, 3, 16, yk.TYPE_INT32_T),
              oracle.type_create_vector(4096, 3, 16, yk.TYPE_INT32_T)) for _ in range(3)]
    size = prod.size(types[0][0])
    ext = prod.extent(types[0][0])[1]
    typed = fill(rng, 4 * ext + 64, "int32")
    tg = dev_copy(cuda, typed)
    expect = np.zeros(size * 4, dtype=np.uint8)
    oracle.pack(typed.ctypes.data, 4, types[0][1], 0, expect.ctypes.data, size * 4)
    before = prod.autotune_stats()
    for i in range(40):
        outs = [cuda.zeros(size * 4, dtype=cuda.uint8, device="cuda") for _ in types]
        prod.pup_batch(prod.batch_array([yk.pack_op(tg.data_ptr(), 4, tp, 0, o.data_ptr(), size * 4)
                                         for (tp, _), o in zip(types, outs)]))
        cuda.cuda.synchronize()
        for o in outs:
            assert np.array_equal(host_of(cuda, o), expect), i
    after = prod.autotune_stats()
    assert after["decided"] > before["decided"]
    for tp, to in types:
        prod.type_free(tp)
        oracle.type_free(to)
