"""GPU: the segmented packs of the reference's pack test (test/pack/pack.c options
-segments, -ordering normal/reverse/random and -overlap none/regular/irregular, with
operators) restated.  The packed range is cut into segments at builtin boundaries.
The segments are packed, then unpacked, in normal, reverse or random order, each
optionally running into the next one (by one element, or by a random part of it).  The
same call sequence on the oracle gives the same bytes, including the operators applied
twice where segments overlap.

Tolerance: byte-identical.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import Pair, assert_same_bytes, dev_copy, fill, host_of, segments
from typegen import BASE, VALID_OPS, Gen, footprint

pytestmark = pytest.mark.gpu

ORDERINGS = ["normal", "reverse", "random"]
OVERLAPS = ["none", "regular", "irregular"]
BASES = ["int8", "int16", "int32", "int64", "float", "double", "c_complex"]


def plan_segments(rng, total, unit, ordering, overlap):
    segs = segments(rng, total, unit, 12)
    out = []
    for i, (s, n) in enumerate(segs):
        if overlap != "none" and i + 1 < len(segs):
            nxt = segs[i + 1][1]
            extra = unit if overlap == "regular" else int(rng.integers(0, nxt // unit + 1)) * unit
            n = min(total - s, n + extra)
        out.append((s, n))
    if ordering == "reverse":
        out.reverse()
    elif ordering == "random":
        out = [out[i] for i in rng.permutation(len(out))]
    return out


@pytest.mark.parametrize("overlap", OVERLAPS)
@pytest.mark.parametrize("ordering", ORDERINGS)
def test_segment_orders_match_oracle(cuda, prod, oracle, ordering, overlap):
    k = ORDERINGS.index(ordering) * len(OVERLAPS) + OVERLAPS.index(overlap)
    rng = np.random.default_rng(700 + k)
    g = Gen(oracle, 13000 + k, max_depth=3)
    for i in range(10):
        base = BASES[i % len(BASES)]
        unit = BASE[base][1]
        pair = Pair(prod, oracle, g.gen(base))
        count = int(rng.integers(1, 6))
        lo, hi, size = footprint(oracle, pair.ho, count)
        total = size * count
        op = yk.OP_NAMES[str(rng.choice(VALID_OPS[base]))]
        typed = fill(rng, hi - lo + 64, base)
        packed = fill(rng, total + 64, base)
        dst = fill(rng, hi - lo + 64, base)
        t_o, p_o, d_o = typed.copy(), packed.copy(), dst.copy()
        t_g, p_g, d_g = dev_copy(cuda, typed), dev_copy(cuda, packed), dev_copy(cuda, dst)
        plan = plan_segments(rng, total, unit, ordering, overlap)
        for s, n in plan:
            ao = oracle.pack(t_o.ctypes.data + 32 - lo, count, pair.ho, s, p_o.ctypes.data + s, n, op=op)
            ap = prod.pack(t_g.data_ptr() + 32 - lo, count, pair.hp, s, p_g.data_ptr() + s, n, op=op)
            assert ao == ap, ("pack", s, n, ao, ap)
        for s, n in plan:
            ao = oracle.unpack(p_o.ctypes.data + s, n, d_o.ctypes.data + 32 - lo, count, pair.ho, s, op=op)
            ap = prod.unpack(p_g.data_ptr() + s, n, d_g.data_ptr() + 32 - lo, count, pair.hp, s, op=op)
            assert ao == ap, ("unpack", s, n, ao, ap)
        cuda.cuda.synchronize()
        assert_same_bytes(host_of(cuda, p_g), p_o, f"packed {ordering}/{overlap}", base)
        assert_same_bytes(host_of(cuda, d_g), d_o, f"unpacked {ordering}/{overlap}", base)
        pair.free()
    g.free()
