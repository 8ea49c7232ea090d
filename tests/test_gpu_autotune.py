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


def test_operator_and_hindexed_grids_are_tuned_and_exact(cuda, prod, oracle):
    """the typed-operator kernel (SUM into a strided target) and the hindexed kernel take
    their grid caps from the autotuner; every launch gives the oracle's bytes"""
    rng = np.random.default_rng(5)
    vp, vo = (y.type_create_hvector(1 << 16, 2, 24, yk.TYPE_DOUBLE) for y in (prod, oracle))
    nb = 40000
    blens = rng.integers(1, 40, nb)
    displs = (np.cumsum(blens + rng.integers(0, 9, nb)) - blens) * 4
    perm = rng.permutation(nb)
    hp, ho = (y.type_create_hindexed(blens[perm].tolist(), displs[perm].tolist(), yk.TYPE_INT32_T)
              for y in (prod, oracle))
    before = prod.autotune_stats()
    for (tp, to, base, op) in ((vp, vo, "double", yk.OP_SUM), (hp, ho, "int32", yk.OP_REPLACE)):
        lb, text = prod.true_extent(tp)
        n = prod.size(tp)
        typed0 = fill(rng, lb + text, base)
        packed0 = fill(rng, n, base)
        exp = typed0.copy()
        oracle.unpack(packed0.ctypes.data, n, exp.ctypes.data, 1, to, 0, op=op)
        pg = dev_copy(cuda, packed0)
        for i in range(40):
            tg = dev_copy(cuda, typed0)
            prod.unpack(pg.data_ptr(), n, tg.data_ptr(), 1, tp, 0, op=op)
            cuda.cuda.synchronize()
            assert np.array_equal(host_of(cuda, tg), exp), (base, i)
    after = prod.autotune_stats()
    assert after["decided"] >= before["decided"] + 2
    for y, t in ((prod, vp), (prod, hp), (oracle, vo), (oracle, ho)):
        y.type_free(t)


_PERSIST_CHILD = r"""
import ctypes, json, sys
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[2])
import numpy as np, torch
import yaksa_gb300 as yk
from conftest import _ensure_product
y = yk.Yaksa(_ensure_product()); y.init()
t = y.type_create_hvector(1 << 17, 1, 64, yk.TYPE_DOUBLE)
src = torch.zeros((1 << 17) * 64, dtype=torch.uint8, device="cuda")
out = torch.zeros(1 << 20, dtype=torch.uint8, device="cuda")
for _ in range(int(sys.argv[3])):
    y.pack(src.data_ptr(), 1, t, 0, out.data_ptr(), 1 << 20)
torch.cuda.synchronize()
print(json.dumps(y.autotune_stats()))
"""


def test_decisions_persist_across_processes(cuda, tmp_path):
    """with YAKSA_GB300_TUNE_FILE set, a process appends each decided shape class to the
    file, and the next process on the same kind of GPU starts with that class decided:
    its launches of the shape are not timed"""
    import json
    import os
    import subprocess
    import sys
    tests = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(tests)
    f = tmp_path / "tune.txt"
    env = dict(os.environ, YAKSA_GB300_TUNE_FILE=str(f))

    def child(n):
        r = subprocess.run([sys.executable, "-c", _PERSIST_CHILD, root, tests, str(n)], env=env,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-3000:]
        return json.loads(r.stdout.strip().splitlines()[-1])

    first = child(40)
    assert first["decided"] >= 1 and first["probes"] > 0, first
    assert f.exists() and f.read_text().strip(), "no decision written"
    second = child(5)
    assert second["decided"] == second["classes"] and second["probes"] == 0, second
