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


def test_server_idle_exit_is_prompt(cuda, prod):
    """A device-wide synchronize waits for resident CTAs, which leave after 2 ms without
    work by the GPU's timer: it returns well before the old 4000-poll bound (about
    50 ms at the measured 12.5 us per idle poll), every time."""
    srv = yk.Server(prod)
    t = prod.type_create_hvector(1 << 15, 4, 128, yk.TYPE_DOUBLE)    # 1 MiB packed
    src = cuda.randn((1 << 15) * 16, dtype=cuda.float64, device="cuda")
    out = cuda.zeros(1 << 17, dtype=cuda.float64, device="cuda")
    cuda.cuda.synchronize()
    waits = []
    for rep in range(5):
        tk = submit_all(srv, [yk.pack_op(src.data_ptr(), 1, t, 0, out.data_ptr(), 1 << 20)])[0]
        srv.wait(tk)
        t0 = time.perf_counter()
        cuda.cuda.synchronize()
        waits.append(time.perf_counter() - t0)
    assert cuda.equal(out, src.view(-1, 16)[:, :4].reshape(-1))
    assert max(waits) < 0.02, waits
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


def test_server_large_requests_split(cuda, prod, oracle):
    """Requests of 2-4 MiB from four families (hvector, lognormal hindexed, struct,
    sorted overlapping blocks unpacked with MAX) submitted together: each is split into
    many work items claimed across the lanes, and every byte matches the oracle."""
    rng = np.random.default_rng(21)
    nb = 20000
    blens = np.clip(np.round(np.exp(np.log(16) + rng.standard_normal(nb))), 1, 4096).astype(np.int64)
    gaps = rng.integers(0, 64, nb)
    order = rng.permutation(nb)
    starts = np.cumsum(blens[order] + gaps) - blens[order]
    displs = np.empty(nb, dtype=np.int64)
    displs[order] = starts * 4
    offs = np.sort(rng.integers(0, (1 << 16) * 8, 1 << 16)).astype(np.int64)
    specs = [
        ("double", 1, lambda y: y.type_create_hvector(1 << 17, 4, 128, yk.TYPE_DOUBLE), 0, yk.OP_REPLACE),
        ("int32", 1, lambda y: y.type_create_hindexed_arrays(nb, blens.ctypes.data, displs.ctypes.data,
                                                             yk.TYPE_INT32_T), 1, yk.OP_REPLACE),
        ("float", 200000, lambda y: y.type_create_resized(
            y.type_create_struct([1, 3], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT]), 0, 32), 0, yk.OP_REPLACE),
        ("int64", 1, lambda y: y.type_create_indexed_block_array(1 << 16, 8, offs.ctypes.data,
                                                                 yk.TYPE_INT64_T), 1, yk.OP_MAX),
    ]
    srv = yk.Server(prod)
    reqs, ops = [], []
    for base, count, mk, kind, op in specs:
        tp, to = mk(prod), mk(oracle)
        lo, hi, size = footprint(oracle, to, count)
        r = dict(tp=tp, to=to, lo=lo, count=count, n=size * count, kind=kind, op=op, base=base,
                 typed=fill(rng, hi - lo + 64, base), packed=fill(rng, size * count + 64, base))
        r["t_g"], r["p_g"] = dev_copy(cuda, r["typed"]), dev_copy(cuda, r["packed"])
        tpp = r["t_g"].data_ptr() + 32 - lo
        ops.append(yk.pack_op(tpp, count, tp, 0, r["p_g"].data_ptr(), r["n"], op=op) if kind == 0 else
                   yk.unpack_op(r["p_g"].data_ptr(), r["n"], tpp, count, tp, 0, op=op))
        reqs.append(r)
    assert min(r["n"] for r in reqs) >= 2 << 20
    for t in submit_all(srv, ops):
        srv.wait(t)
    cuda.cuda.synchronize()
    for r, o in zip(reqs, ops):
        th, ph = r["typed"].copy(), r["packed"].copy()
        tpo = th.ctypes.data + 32 - r["lo"]
        if r["kind"] == 0:
            a = oracle.pack(tpo, r["count"], r["to"], 0, ph.ctypes.data, r["n"], op=r["op"])
        else:
            a = oracle.unpack(ph.ctypes.data, r["n"], tpo, r["count"], r["to"], 0, op=r["op"])
        assert o.actual == a == r["n"]
        assert_same_bytes(host_of(cuda, r["p_g"]), ph, "server packed", r["base"])
        assert_same_bytes(host_of(cuda, r["t_g"]), th, "server typed", r["base"])
        prod.type_free(r["tp"])
        oracle.type_free(r["to"])
    srv.destroy()


SB_BASES = [("int8", yk.TYPE_INT8_T), ("int16", yk.TYPE_INT16_T), ("int32", yk.TYPE_INT32_T),
            ("int64", yk.TYPE_INT64_T), ("float", yk.TYPE_FLOAT), ("double", yk.TYPE_DOUBLE),
            ("c_complex", yk.TYPE_C_COMPLEX), ("c_double_complex", yk.TYPE_C_DOUBLE_COMPLEX)]


@pytest.mark.parametrize("base,h", SB_BASES)
@pytest.mark.parametrize("bl", [8, 3])
def test_server_sorted_block_items(cuda, prod, oracle, base, h, bl):
    """Unpacks into overlapping sorted blocks through the server, for every base type of
    its sorted-block items and each of SUM, PROD, MAX, MIN and REPLACE that the type has:
    blocks of 8 elements (a power of two in bytes: the per-lane item with 32-bit offsets,
    or the L2-reduction item for 4- and 8-byte integers) and of 3 (the generic item).
    About four blocks cover each element; the requests, each cut into many items, run
    together, and each matches the oracle."""
    rng = np.random.default_rng(bl * 100 + h)
    nblk = 1 << 14
    offs = np.sort(rng.integers(0, nblk * bl // 4, nblk)).astype(np.int64)
    names = [o for o in ("sum", "prod", "max", "min", "replace") if o in VALID_OPS[base]]
    tp = prod.type_create_indexed_block_array(nblk, bl, offs.ctypes.data, h)
    to = oracle.type_create_indexed_block_array(nblk, bl, offs.ctypes.data, h)
    lo, hi, size = footprint(oracle, to, 1)
    srv = yk.Server(prod)
    reqs, ops = [], []
    for name in names:
        r = dict(op=yk.OP_NAMES[name], typed=fill(rng, hi - lo + 64, base),
                 packed=fill(rng, size + 64, base))
        r["t_g"], r["p_g"] = dev_copy(cuda, r["typed"]), dev_copy(cuda, r["packed"])
        ops.append(yk.unpack_op(r["p_g"].data_ptr(), size, r["t_g"].data_ptr() + 32 - lo, 1, tp, 0,
                                op=r["op"]))
        reqs.append(r)
    for t in submit_all(srv, ops):
        srv.wait(t)
    cuda.cuda.synchronize()
    for r, o, name in zip(reqs, ops, names):
        th = r["typed"].copy()
        a = oracle.unpack(r["packed"].ctypes.data, size, th.ctypes.data + 32 - lo, 1, to, 0, op=r["op"])
        assert o.actual == a == size
        assert_same_bytes(host_of(cuda, r["t_g"]), th, f"server sorted blocks {base} {name} bl {bl}")
    srv.destroy()
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("env", [{"YAKSA_GB300_SERVER_ITEM_KIB": "16", "YAKSA_GB300_SERVER_MIN_ITEMS": "0"},
                                 {"YAKSA_GB300_SERVER_MIN_ITEMS": "1024"}])
def test_server_item_sizes(cuda, env):
    """The server tests again, in a child process, with 16 KiB items or at least 1024
    items per request: many items per request spread over every claim lane."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-p", "no:cacheprovider",
                        os.path.join(here, "test_gpu_server.py"), "-k", "not item_sizes"],
                       env=dict(os.environ, **env), capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]


def test_server_tune_decides_item_cuts_and_stays_exact(cuda, prod, oracle):
    """yaksa_gb300_server_tune times every candidate item cut of each class of 256 KiB and
    more (hvector and hindexed packs, a strided SUM unpack) with the request alone on the
    server, decides each class once, and later submissions -- cut the decided way --
    give the oracle's bytes; a second call finds every class decided"""
    rng = np.random.default_rng(31)
    nb = 30000
    blens = rng.integers(1, 40, nb)
    displs = (np.cumsum(blens + rng.integers(0, 9, nb)) - blens) * 4
    perm = rng.permutation(nb)
    specs = [("hvector", lambda y: y.type_create_hvector(1 << 16, 4, 64, yk.TYPE_DOUBLE), "double",
              yk.OP_REPLACE, 0),
             ("hindexed", lambda y: y.type_create_hindexed(blens[perm].tolist(), displs[perm].tolist(),
                                                          yk.TYPE_INT32_T), "int32", yk.OP_REPLACE, 0),
             ("strided_sum", lambda y: y.type_create_hvector(1 << 15, 8, 96, yk.TYPE_DOUBLE), "double",
              yk.OP_SUM, 1)]
    srv = yk.Server(prod, ring_requests=64)
    reqs = []
    for name, mk, base, op, kind in specs:
        tp, to = mk(prod), mk(oracle)
        lb, text = prod.true_extent(tp)
        n = prod.size(tp)
        assert n >= 256 << 10
        typed, packed = fill(rng, lb + text, base), fill(rng, n, base)
        reqs.append(dict(tp=tp, to=to, lb=lb, n=n, typed=typed, packed=packed, op=op, kind=kind))

    def ops_of(bufs):
        out = []
        for r, (tg, pg) in zip(reqs, bufs):
            if r["kind"] == 0:
                out.append(yk.pack_op(tg.data_ptr() - r["lb"], 1, r["tp"], 0, pg.data_ptr(), r["n"]))
            else:
                out.append(yk.unpack_op(pg.data_ptr(), r["n"], tg.data_ptr() - r["lb"], 1, r["tp"], 0,
                                        op=r["op"]))
        return prod.batch_array(out)

    scratch = [(dev_copy(cuda, r["typed"]), dev_copy(cuda, r["packed"])) for r in reqs]
    before = prod.autotune_stats()["decided"]
    decided = srv.tune(ops_of(scratch))
    assert decided == len(reqs)
    assert prod.autotune_stats()["decided"] == before + len(reqs)
    assert srv.tune(ops_of(scratch)) == 0
    # submissions after the decision: bytes against the oracle
    bufs = [(dev_copy(cuda, r["typed"]), dev_copy(cuda, r["packed"])) for r in reqs]
    tickets = submit_all(srv, list(ops_of(bufs)))
    for t in tickets:
        srv.wait(t)
    for r, (tg, pg) in zip(reqs, bufs):
        th, ph = r["typed"].copy(), r["packed"].copy()
        if r["kind"] == 0:
            oracle.pack(th.ctypes.data - r["lb"], 1, r["to"], 0, ph.ctypes.data, r["n"])
        else:
            oracle.unpack(ph.ctypes.data, r["n"], th.ctypes.data - r["lb"], 1, r["to"], 0, op=r["op"])
        assert np.array_equal(host_of(cuda, tg), th)
        assert np.array_equal(host_of(cuda, pg), ph)
    srv.destroy()
    for r in reqs:
        prod.type_free(r["tp"])
        oracle.type_free(r["to"])


@pytest.mark.parametrize("fields,count", [
    (([1, 3], [0, 8], ["TYPE_INT64_T", "TYPE_FLOAT"], 32), 300_001),    # 20-byte runs
    (([3, 3], [0, 12], ["TYPE_INT32_T", "TYPE_FLOAT"], 32), 70_013),     # 24-byte runs
    (([1, 7], [0, 8], ["TYPE_INT64_T", "TYPE_FLOAT"], 48), 50_021),      # 36-byte runs
])
def test_server_struct_like_packs(cuda, prod, oracle, fields, count):
    """Packs of struct-like runs (17-47 bytes on 16-byte element starts) through the
    server's warp-staged item: items of whole 32-element groups, a last group of fewer
    than 32 elements, the packed bytes against the oracle."""
    blens, displs, names, extent = fields
    ts = [getattr(yk, n) for n in names]
    sp = prod.type_create_struct(blens, displs, ts)
    so = oracle.type_create_struct(blens, displs, ts)
    tp, to = prod.type_create_resized(sp, 0, extent), oracle.type_create_resized(so, 0, extent)
    rng = np.random.default_rng(count)
    typed = rng.integers(0, 256, count * extent, dtype=np.uint8)
    n = prod.size(tp) * count
    exp = np.zeros(n, dtype=np.uint8)
    oracle.pack(typed.ctypes.data, count, to, 0, exp.ctypes.data, n)
    td = cuda.from_numpy(typed).cuda()
    out = cuda.zeros(n, dtype=cuda.uint8, device="cuda")
    cuda.cuda.synchronize()
    srv = yk.Server(prod)
    try:
        tk = submit_all(srv, [yk.pack_op(td.data_ptr(), count, tp, 0, out.data_ptr(), n)])[0]
        srv.wait(tk)
        assert srv.stats()["items"] >= 2
        assert np.array_equal(out.cpu().numpy(), exp)
    finally:
        srv.destroy()
    for y, t in ((prod, tp), (prod, sp), (oracle, to), (oracle, so)):
        y.type_free(t)
