"""GPU: the persistent-kernel request server gives the oracle's bytes for every
request, whether it runs alone or mixed with many others, including requests that
arrive while the resident CTAs are busy, after they left on idle, operators, and
ordered (overlapping) unpacks.

Tolerance: byte-identical (REPLACE and integer operators; floats as in
test_gpu_parity: NaN payloads are not pinned, no input here produces NaN).
"""
import time

import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import Pair, assert_same_bytes, dev_copy, fill, host_of
from typegen import VALID_OPS, Gen, footprint

pytestmark = pytest.mark.gpu


def make_requests(cuda, prod, oracle, seed, n, ops=True):
    rng = np.random.default_rng(seed)
    bases = ["int32", "double", "int8", "float", "int64", "c_complex", "int16"]
    g = Gen(oracle, 11000 + seed, max_depth=3)
    reqs = []
    for i in range(n):
        base = bases[i % len(bases)]
        pair = Pair(prod, oracle, g.gen(base))
        count = int(rng.integers(1, 5))
        lo, hi, size = footprint(oracle, pair.ho, count)
        opname = rng.choice(VALID_OPS[base]) if ops and i % 3 == 0 else "replace"
        r = dict(pair=pair, count=count, lo=lo, size=size, base=base, op=yk.OP_NAMES[opname],
                 kind=int(rng.integers(0, 2)), typed=fill(rng, hi - lo + 64, base),
                 packed=fill(rng, size * count + 64, base))
        r["t_g"], r["p_g"] = dev_copy(cuda, r["typed"]), dev_copy(cuda, r["packed"])
        reqs.append(r)
    return g, reqs


def oracle_apply(oracle, r):
    th, ph = r["typed"].copy(), r["packed"].copy()
    n = r["size"] * r["count"]
    to = th.ctypes.data + 32 - r["lo"]
    if r["kind"] == 0:
        a = oracle.pack(to, r["count"], r["pair"].ho, 0, ph.ctypes.data, n, op=r["op"])
    else:
        a = oracle.unpack(ph.ctypes.data, n, to, r["count"], r["pair"].ho, 0, op=r["op"])
    return th, ph, a


def op_of(r):
    n = r["size"] * r["count"]
    tp = r["t_g"].data_ptr() + 32 - r["lo"]
    if r["kind"] == 0:
        return yk.pack_op(tp, r["count"], r["pair"].hp, 0, r["p_g"].data_ptr(), n, op=r["op"])
    return yk.unpack_op(r["p_g"].data_ptr(), n, tp, r["count"], r["pair"].hp, 0, op=r["op"])


def submit_all(srv, ops):
    tickets = []
    for o in ops:
        for _ in range(100000):
            t = srv.submit(o)
            if t is not None:
                break
            srv.progress()
        assert t is not None
        tickets.append(t)
    return tickets


@pytest.mark.parametrize("seed", range(3))
def test_server_matches_oracle(cuda, prod, oracle, seed):
    g, reqs = make_requests(cuda, prod, oracle, seed, 40)
    srv = yk.Server(prod, ring_requests=64)
    ops = [op_of(r) for r in reqs]
    tickets = submit_all(srv, ops)
    for t in tickets:
        srv.wait(t)
    cuda.cuda.synchronize()
    for r, o in zip(reqs, ops):
        th, ph, a = oracle_apply(oracle, r)
        assert o.actual == a
        assert_same_bytes(host_of(cuda, r["p_g"]), ph, "server packed", r["base"])
        assert_same_bytes(host_of(cuda, r["t_g"]), th, "server typed", r["base"])
        r["pair"].free()
    srv.destroy()
    g.free()


def test_server_alone_equals_mixed(cuda, prod, oracle):
    """Each request's result is the same submitted alone or inside a stream of others."""
    g, reqs = make_requests(cuda, prod, oracle, 7, 24)
    srv = yk.Server(prod)
    # alone, one at a time
    alone = []
    for r in reqs:
        t = submit_all(srv, [op_of(r)])[0]
        srv.wait(t)
        alone.append((host_of(cuda, r["p_g"]).copy(), host_of(cuda, r["t_g"]).copy()))
        r["t_g"].copy_(cuda.from_numpy(r["typed"]))
        r["p_g"].copy_(cuda.from_numpy(r["packed"]))
    cuda.cuda.synchronize()
    # mixed: all in flight together
    tickets = submit_all(srv, [op_of(r) for r in reqs])
    for t in tickets:
        srv.wait(t)
    for r, (pa, ta) in zip(reqs, alone):
        assert np.array_equal(host_of(cuda, r["p_g"]), pa)
        assert np.array_equal(host_of(cuda, r["t_g"]), ta)
        r["pair"].free()
    srv.destroy()
    g.free()


def test_server_idle_exit_and_relaunch(cuda, prod, oracle):
    """Resident CTAs leave after idling; later submissions relaunch them."""
    srv = yk.Server(prod)
    t = prod.type_create_hvector(1024, 4, 128, yk.TYPE_DOUBLE)
    src = cuda.randn(1024 * 16, dtype=cuda.float64, device="cuda")
    for rep in range(3):
        out = cuda.zeros(4096, dtype=cuda.float64, device="cuda")
        tk = submit_all(srv, [yk.pack_op(src.data_ptr(), 1, t, 0, out.data_ptr(), 32768)])[0]
        srv.wait(tk)
        assert cuda.equal(out, src.view(1024, 16)[:, :4].reshape(-1))
        time.sleep(0.1)         # longer than the idle bound
    st = srv.stats()
    assert st["relaunches"] >= 2 and st["idle_exits"] >= 1, st
    srv.destroy()
    prod.type_free(t)


def test_server_admission_budget(cuda, prod, oracle):
    """A byte budget smaller than the queue refuses admission until requests finish."""
    srv = yk.Server(prod, ring_requests=8, budget_bytes=1 << 20)
    t = prod.type_create_hvector(1 << 16, 4, 32, yk.TYPE_FLOAT)    # 1 MiB packed
    src = cuda.randn((1 << 16) * 8, device="cuda")
    outs = [cuda.zeros(1 << 18, device="cuda") for _ in range(6)]
    tickets, refused = [], 0
    for o in outs:
        op = yk.pack_op(src.data_ptr(), 1, t, 0, o.data_ptr(), 1 << 20)
        while True:
            tk = srv.submit(op)
            if tk is not None:
                break
            refused += 1
            srv.progress()
        tickets.append(tk)
    for tk in tickets:
        srv.wait(tk)
    ref = src.view(-1, 8)[:, :4].reshape(-1)
    for o in outs:
        assert cuda.equal(o, ref)
    # a request larger than the budget is still admitted when nothing else is in flight
    big = yk.pack_op(src.data_ptr(), 1, t, 0, outs[0].data_ptr(), 1 << 20)
    srv2 = yk.Server(prod, ring_requests=8, budget_bytes=1024)
    tk = submit_all(srv2, [big])[0]
    srv2.wait(tk)
    srv2.destroy()
    srv.destroy()
    prod.type_free(t)
