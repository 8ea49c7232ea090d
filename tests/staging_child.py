"""Child process of test_gpu_staging.py: runs packs and unpacks whose host buffers the
library must stage (YAKSA_GB300_HOST_DIRECT=0 in the environment, set by the parent
before the library starts), and prints one JSON line with a verdict per case.

Every case compares the product's bytes with the oracle's on the same inputs.  The
ring is made small by the parent (YAKSA_GB300_STAGE_SLABS, YAKSA_GB300_STAGE_SLAB_KIB)
so that requests span many chunks and wrap around the ring.
"""
import ctypes
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

import yaksa_gb300 as yk  # noqa: E402
from conftest import _ensure_oracle, _ensure_product  # noqa: E402


def main():
    prod = yk.Yaksa(_ensure_product())
    orc = yk.Yaksa(_ensure_oracle())
    prod.init()
    orc.init()
    rng = np.random.default_rng(41)
    out = {}

    def both(ctor, *a):
        return getattr(prod, ctor)(*a), getattr(orc, ctor)(*a)

    def bounds(t, count):
        lb, text = prod.true_extent(t)
        ext = prod.extent(t)[1]
        return min(lb, lb + (count - 1) * ext), max(lb + text, lb + text + (count - 1) * ext)

    def host(arr, pinned):
        """a host buffer holding arr's bytes: pageable numpy, or pinned torch memory"""
        if pinned:
            t = torch.from_numpy(arr.copy()).pin_memory()
            return t, t.data_ptr(), lambda: t.numpy().copy()
        a = arr.copy()
        return a, a.ctypes.data, lambda: a.copy()

    def dev(arr):
        t = torch.from_numpy(arr.copy()).cuda()
        torch.cuda.synchronize()
        return t, t.data_ptr(), lambda: t.cpu().numpy()

    def case(name, tp, to, count, direction, typed_where, packed_where, op=yk.OP_REPLACE,
             kind=np.uint8, mode="wait"):
        lo, hi = bounds(tp, count)
        n = prod.size(tp) * count
        typed0 = rng.integers(0, 256, hi - lo, dtype=np.uint8)
        packed0 = rng.integers(0, 256, n, dtype=np.uint8)
        if kind is not np.uint8:
            assert (hi - lo) % 8 == 0 and n % 8 == 0
            typed0 = rng.standard_normal((hi - lo) // 8).view(np.uint8)
            packed0 = rng.standard_normal(n // 8).view(np.uint8)
        mk = {"dev": dev, "host": lambda a: host(a, False), "pinned": lambda a: host(a, True)}
        tkeep, tptr, tget = mk[typed_where](typed0)
        pkeep, pptr, pget = mk[packed_where](packed0)
        th, ph = typed0.copy(), packed0.copy()
        if direction == "pack":
            a = orc.pack(th.ctypes.data - lo, count, to, 0, ph.ctypes.data, n, op=op)
            if mode == "stream":
                h = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
                got = prod.pack_stream(tptr - lo, count, tp, 0, pptr, n, ctypes.addressof(h), op=op)
                torch.cuda.current_stream().synchronize()
            else:
                got, req = prod.ipack(tptr - lo, count, tp, 0, pptr, n, op=op)
                prod.wait(req)
        else:
            a = orc.unpack(ph.ctypes.data, n, th.ctypes.data - lo, count, to, 0, op=op)
            if mode == "stream":
                h = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
                got = prod.unpack_stream(pptr, n, tptr - lo, count, tp, 0, ctypes.addressof(h), op=op)
                torch.cuda.current_stream().synchronize()
            else:
                got, req = prod.iunpack(pptr, n, tptr - lo, count, tp, 0, op=op)
                prod.wait(req)
        ok = got == a and np.array_equal(tget(), th) and np.array_equal(pget(), ph)
        out[name] = bool(ok)

    s0 = prod.stats()
    # hvector of doubles, 5 MiB packed: many 64 KiB chunks, packed side staged
    vp, vo = both("type_create_hvector", 163840, 4, 48, yk.TYPE_DOUBLE)
    case("pack_packed_host", vp, vo, 1, "pack", "dev", "host")
    case("unpack_packed_host", vp, vo, 1, "unpack", "dev", "host")
    case("pack_packed_pinned", vp, vo, 1, "pack", "dev", "pinned")
    case("pack_stream_packed_host", vp, vo, 1, "pack", "dev", "host", mode="stream")
    # typed side staged: 2000 elements of about 3 KiB span, chunks of whole elements
    wp, wo = both("type_create_hvector", 64, 4, 48, yk.TYPE_DOUBLE)
    case("pack_typed_host", wp, wo, 2000, "pack", "host", "dev")
    case("unpack_typed_host", wp, wo, 2000, "unpack", "host", "dev")
    case("pack_both_host", wp, wo, 2000, "pack", "host", "host")
    case("unpack_both_host", wp, wo, 2000, "unpack", "pinned", "host")
    case("unpack_sum_typed_host", wp, wo, 2000, "unpack", "host", "dev", op=yk.OP_SUM, kind=np.float64)
    # count > 1 of a small element: chunks of whole elements when the typed side is staged
    sp, so = both("type_create_struct", [1, 3], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT])
    rp, ro = prod.type_create_resized(sp, 0, 32), orc.type_create_resized(so, 0, 32)
    case("struct_pack_typed_host", rp, ro, 100000, "pack", "host", "dev")
    case("struct_unpack_both_host", rp, ro, 100000, "unpack", "host", "host")
    # elements that overlap by half (8 doubles at a 32-byte extent), unpacked with SUM into
    # a staged typed buffer: the typed spans of consecutive chunks overlap, so each
    # chunk's copy in must follow the previous chunk's copy out
    cp, co = both("type_create_contig", 8, yk.TYPE_DOUBLE)
    ip, io = prod.type_create_resized(cp, 0, 32), orc.type_create_resized(co, 0, 32)
    case("overlap_sum_typed_host", ip, io, 20000, "unpack", "host", "dev", op=yk.OP_SUM, kind=np.float64)
    case("overlap_replace_both_host", ip, io, 20000, "unpack", "host", "host")
    # overlapping blocks of one indexed_block level under int64 SUM: the typed span is
    # staged into device memory, where the L2-reduction form folds the blocks in
    qoffs = sorted(rng.integers(0, 3000, 4000).tolist())
    iq, iqo = both("type_create_indexed_block", 8, qoffs, yk.TYPE_INT64_T)
    red0 = ctypes.c_ulonglong(0)
    prod.lib.yaksa_gb300_debug_l2_reduce(-1, ctypes.byref(red0))
    case("overlap_int_sum_typed_host", iq, iqo, 1, "unpack", "host", "dev", op=yk.OP_SUM)
    red1 = ctypes.c_ulonglong(0)
    prod.lib.yaksa_gb300_debug_l2_reduce(-1, ctypes.byref(red1))
    out["l2_reduce_on_staged_span"] = red1.value > red0.value
    # hindexed in shuffled order with gaps
    nb = 40000
    blens = rng.integers(1, 40, nb)
    displs = (np.cumsum(blens + rng.integers(0, 9, nb)) - blens) * 4
    perm = rng.permutation(nb)
    hp, ho = both("type_create_hindexed", blens[perm].tolist(), displs[perm].tolist(), yk.TYPE_INT32_T)
    case("hindexed_pack_packed_host", hp, ho, 1, "pack", "dev", "host")
    case("hindexed_unpack_both_host", hp, ho, 1, "unpack", "host", "host")
    # one element's span (1 MiB) larger than a slab: the stream-ordered one-off path
    bp, bo = both("type_create_hvector", 512, 2, 2048, yk.TYPE_FLOAT)
    case("oversize_pack_typed_host", bp, bo, 1, "pack", "host", "dev")
    case("oversize_unpack_typed_host", bp, bo, 1, "unpack", "host", "host")

    # more requests in flight than the ring holds: 40 nonblocking packs into host buffers
    src = torch.from_numpy(rng.integers(0, 256, 163840 * 48, dtype=np.uint8)).cuda()
    torch.cuda.synchronize()
    n = prod.size(vp)
    outs = [np.zeros(n, dtype=np.uint8) for _ in range(40)]
    reqs = [prod.ipack(src.data_ptr(), 1, vp, 0, o.ctypes.data, n)[1] for o in outs]
    for r in reqs:
        prod.wait(r)
    ref = np.zeros(n, dtype=np.uint8)
    srch = src.cpu().numpy()
    orc.pack(srch.ctypes.data, 1, vo, 0, ref.ctypes.data, n)
    out["many_in_flight"] = all(np.array_equal(o, ref) for o in outs)

    s1 = prod.stats()
    out["staged_calls"] = s1["staged_calls"] - s0["staged_calls"]
    out["direct_calls"] = s1["direct_calls"] - s0["direct_calls"]
    for y in (prod, orc):
        for t in ((vp, wp, sp, rp, cp, ip, iq, hp, bp) if y is prod else
                  (vo, wo, so, ro, co, io, iqo, ho, bo)):
            y.type_free(t)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
