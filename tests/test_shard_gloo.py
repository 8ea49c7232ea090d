"""CPU, two and three processes over gloo: the sharding rule of yaksa_gb300_shard splits a pack
between ranks with no exchange on the data path.  Each rank computes its part of the
packed range with the product's host-side helper, packs that part (the oracle does the
byte moving, as there is no GPU here), and the parts gathered on rank 0 equal the whole
pack.  The same parts unpacked by each rank into its own buffer rebuild the typed
buffer (for the types whose typemap reaches no byte twice).  Seeded random types of
depth up to 3, counts 1..6, on 2 and 3 ranks.
"""
import ctypes
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, results):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import yaksa_gb300 as yk
    from conftest import _ensure_oracle, _ensure_product
    from typegen import Gen, build, footprint
    from helpers import fill

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    prod = yk.Yaksa(_ensure_product())
    prod.init()
    oracle = yk.Yaksa(_ensure_oracle())
    oracle.init()
    ok = True
    n_checked = 0
    for seed in range(8):
        g = Gen(oracle, 600 + seed, max_depth=3)
        base = ["int32", "double", "int8", "float", "short_int", "c_complex"][seed % 6]
        r = g.gen(base)
        kp, ko = [], []
        hp, ho = build(prod, r, kp), build(oracle, r, ko)
        count = 1 + seed % 6
        lo, hi, size = footprint(oracle, ho, count)
        total = size * count
        rng = np.random.default_rng(seed)
        typed = fill(rng, hi - lo + 64, base)      # the same on every rank (same seed)
        off, n = prod.shard(hp, count, rank, world)
        part = np.zeros(max(n, 1), dtype=np.uint8)
        got = oracle.pack(typed.ctypes.data + 32 - lo, count, ho, off, part.ctypes.data, n)
        ok &= got == n
        # gather (offset, part) on every rank: parts differ in size, so pad to the largest
        sizes = [torch.zeros(2, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(sizes, torch.tensor([off, n], dtype=torch.int64))
        width = max(int(s[1]) for s in sizes) or 1
        buf = torch.zeros(width, dtype=torch.uint8)
        buf[:n] = torch.from_numpy(part[:n])
        parts = [torch.zeros(width, dtype=torch.uint8) for _ in range(world)]
        dist.all_gather(parts, buf)
        whole = np.zeros(total, dtype=np.uint8)
        covered = 0
        for s, p in zip(sizes, parts):
            o, k = int(s[0]), int(s[1])
            ok &= o == covered                     # the parts tile the range in order
            whole[o:o + k] = p[:k].numpy()
            covered += k
        ok &= covered == total
        expect = np.zeros(total, dtype=np.uint8)
        oracle.pack(typed.ctypes.data + 32 - lo, count, ho, 0, expect.ctypes.data, total)
        ok &= bool(np.array_equal(whole, expect))
        # unpack: each rank writes its part into its own copy; summing the ranks'
        # changes rebuilds the one-shot unpack when the parts touch disjoint typed
        # bytes, i.e. for types whose typemap reaches no byte twice (an overlapping
        # type keeps the reference's last-writer order only within one call)
        offs = np.empty(total, dtype=np.int64)
        om = oracle.lib.yaksa_oracle_byte_offsets
        om.restype = ctypes.c_int
        om.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p]
        ok &= om(ho, count, offs.ctypes.data) == 0
        overlapping = len(np.unique(offs)) < total
        base_buf = fill(rng, hi - lo + 64, base)
        mine = base_buf.copy()
        oracle.unpack(part.ctypes.data, n, mine.ctypes.data + 32 - lo, count, ho, off)
        changed = torch.from_numpy((mine != base_buf).astype(np.uint8))
        vals = torch.from_numpy(np.where(mine != base_buf, mine, 0).astype(np.int64))
        dist.all_reduce(changed)
        dist.all_reduce(vals)
        rebuilt = np.where(changed.numpy() > 0, vals.numpy(), base_buf).astype(np.uint8)
        ref = base_buf.copy()
        oracle.unpack(expect.ctypes.data, total, ref.ctypes.data + 32 - lo, count, ho, 0)
        if not overlapping:
            ok &= int(changed.max()) <= 1
            ok &= bool(np.array_equal(rebuilt, ref))
        n_checked += not overlapping
        for y, keep in ((prod, kp), (oracle, ko)):
            for h in reversed(keep):
                y.type_free(h)
        g.free()
    results[rank] = bool(ok) and n_checked >= 4
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_pack_reassembles(world):
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    results = mgr.dict()
    port = free_port()
    mp.start_processes(worker, args=(world, port, results), nprocs=world, start_method="spawn",
                       join=True)
    assert dict(results) == {r: True for r in range(world)}


def test_shard_edges(prod):
    """Host only: bad ranks are errors, an empty range gives empty parts, and parts end on
    builtin boundaries (a struct of one int8 and one double: 9-byte elements)."""
    import yaksa_gb300 as yk
    t = prod.type_create_struct([1, 1], [0, 8], [yk.TYPE_INT8_T, yk.TYPE_DOUBLE])
    for rank, nranks in ((0, 0), (-1, 2), (2, 2)):
        with pytest.raises(Exception):
            prod.shard(t, 4, rank, nranks)
    assert prod.shard(t, 0, 0, 3) == (0, 0)
    assert prod.shard(yk.TYPE_NULL, 5, 1, 3) == (0, 0)
    for count, nranks in ((1, 2), (1, 7), (5, 3), (1000, 7)):
        total = 9 * count
        parts = [prod.shard(t, count, r, nranks) for r in range(nranks)]
        assert parts[0][0] == 0
        assert sum(n for _, n in parts) == total
        for (o0, n0), (o1, _) in zip(parts, parts[1:]):
            assert o0 + n0 == o1
        for o, _ in parts:
            assert o % 9 in (0, 1)               # the int8 or the double starts here
    prod.type_free(t)
