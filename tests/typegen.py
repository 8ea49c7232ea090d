"""Seeded random datatype recipes for parity tests.

A recipe is a nested tuple describing constructor calls; `build(y, recipe)` replays it
on any library exposing the yaksa C ABI (the GPU engine or the CPU oracle), so both
sides see the same type.  The generator covers every constructor of the reference API
(src/frontend/include/yaksa.h.in:264-402) with positive and negative strides, resized
bounds and structs of mixed base types, in the spirit of the reference's dtpools
generator (test/dtpools) but written for these tests.

Layouts are non-overlapping unless `overlap=True`, so unpack results are defined.
"""
import random

import yaksa_gb300 as yk

# (handle, size, numpy dtype name used to fill buffers)
BASE = {
    "int8": (yk.TYPE_INT8_T, 1, "i1"),
    "int16": (yk.TYPE_INT16_T, 2, "i2"),
    "int32": (yk.TYPE_INT32_T, 4, "i4"),
    "int64": (yk.TYPE_INT64_T, 8, "i8"),
    "uint32": (yk.TYPE_UINT32_T, 4, "u4"),
    "float": (yk.TYPE_FLOAT, 4, "f4"),
    "double": (yk.TYPE_DOUBLE, 8, "f8"),
    "c_complex": (yk.TYPE_C_COMPLEX, 8, "c8"),
    "c_double_complex": (yk.TYPE_C_DOUBLE_COMPLEX, 16, "c16"),
    "bool": (yk.TYPE_BOOL, 1, "bool"),
    "char": (yk.TYPE_CHAR, 1, "i1"),
    "wchar": (yk.TYPE_WCHAR_T, 4, "i4"),
    "short_int": (yk.TYPE_SHORT_INT, 6, None),
    "double_int": (yk.TYPE_DOUBLE_INT, 12, None),
    "float_int": (yk.TYPE_FLOAT_INT, 8, None),
    "2int": (yk.TYPE_2INT, 8, "i4"),
    "long_double": (yk.TYPE_LONG_DOUBLE, 16, None),
}

# operators each base type defines (src/backend/gencomm.py:14-27)
INT_OPS = ["max", "min", "sum", "prod", "land", "band", "lor", "bor", "lxor", "bxor", "replace"]
FLOAT_OPS = ["max", "min", "sum", "prod", "replace"]
COMPLEX_OPS = ["sum", "prod", "replace"]
VALID_OPS = {"int8": INT_OPS, "int16": INT_OPS, "int32": INT_OPS, "int64": INT_OPS,
             "uint32": INT_OPS, "2int": INT_OPS, "float": FLOAT_OPS, "double": FLOAT_OPS,
             "c_complex": COMPLEX_OPS, "c_double_complex": COMPLEX_OPS,
             "bool": ["land", "lor", "lxor", "replace"], "char": ["replace"], "wchar": ["replace"]}


def build(y, r, keep):
    """Instantiate recipe r on Yaksa instance y; intermediate handles go to `keep`."""
    kind = r[0]
    if kind == "builtin":
        return r[1]
    if kind == "struct":
        kids = [build(y, c, keep) for c in r[3]]
        h = y.type_create_struct(r[1], r[2], kids)
    else:
        child = build(y, r[-1], keep)
        if kind == "contig":
            h = y.type_create_contig(r[1], child)
        elif kind == "dup":
            h = y.type_create_dup(child)
        elif kind == "vector":
            h = y.type_create_vector(r[1], r[2], r[3], child)
        elif kind == "hvector":
            h = y.type_create_hvector(r[1], r[2], r[3], child)
        elif kind == "indexed_block":
            h = y.type_create_indexed_block(r[1], r[2], child)
        elif kind == "hindexed_block":
            h = y.type_create_hindexed_block(r[1], r[2], child)
        elif kind == "indexed":
            h = y.type_create_indexed(r[1], r[2], child)
        elif kind == "hindexed":
            h = y.type_create_hindexed(r[1], r[2], child)
        elif kind == "resized":
            h = y.type_create_resized(child, r[1], r[2])
        elif kind == "subarray":
            h = y.type_create_subarray(r[1], r[2], r[3], r[4], child)
        else:
            raise ValueError(kind)
    keep.append(h)
    return h


class Gen:
    """Random recipes; `y` (usually the oracle) answers size/extent queries."""

    def __init__(self, y, seed, max_depth=3, max_size=1 << 14, overlap=False):
        self.y = y
        self.rng = random.Random(seed)
        self.max_depth = max_depth
        self.max_size = max_size
        self.overlap = overlap
        self.keep = []

    def info(self, r):
        h = build(self.y, r, self.keep)
        return self.y.size(h), self.y.extent(h), self.y.true_extent(h)

    def leaf(self, base):
        return ("builtin", BASE[base][0])

    def gen(self, base, depth=None):
        depth = self.max_depth if depth is None else depth
        rng = self.rng
        child = self.leaf(base) if depth <= 1 or rng.random() < 0.25 else self.gen(base, depth - 1)
        size, (lb, ext), (tlb, text) = self.info(child)
        span = max(text, abs(ext), 1)
        budget = max(1, self.max_size // max(size, 1))
        kinds = ["contig", "vector", "hvector", "indexed_block", "hindexed_block", "indexed",
                 "hindexed", "resized", "subarray", "dup", "struct"]
        kind = rng.choice(kinds)
        if kind == "contig":
            return ("contig", rng.randint(1, min(8, budget)), child)
        if kind == "dup":
            return ("dup", child)
        if kind in ("vector", "hvector"):
            count = rng.randint(1, min(8, budget))
            bl = rng.randint(1, max(1, min(4, budget // count)))
            step_elems = bl + rng.randint(0, 3)           # in child extents
            if self.overlap and rng.random() < 0.3:
                step_elems = rng.randint(0, bl)
            sign = -1 if rng.random() < 0.25 else 1
            if kind == "vector":
                return ("vector", count, bl, sign * step_elems, child)
            pad = rng.choice([0, 0, 4, 8, 12])
            return ("hvector", count, bl, sign * (step_elems * abs(ext) + pad), child)
        if kind in ("indexed_block", "hindexed_block", "indexed", "hindexed"):
            count = rng.randint(1, min(8, budget))
            blens = [rng.randint(0 if kind.startswith("h") or kind == "indexed" else 1, 4)
                     for _ in range(count)]
            if kind.endswith("_block"):
                blens = [max(1, blens[0])] * count
            if sum(blens) == 0:
                blens[0] = 1
            displs, pos = [], rng.randint(0, 3)
            for b in blens:
                displs.append(pos)
                pos += b + rng.randint(0, 2)
            if rng.random() < 0.4:                         # permuted block order
                order = list(range(count))
                rng.shuffle(order)
                displs = [displs[i] for i in order]
                blens_perm = [blens[i] for i in order]
                if not kind.endswith("_block"):
                    blens = blens_perm
            if self.overlap and rng.random() < 0.4:
                displs = sorted(rng.randint(0, 2 * count) for _ in range(count))
            if kind.startswith("h"):
                unit = abs(ext) if abs(ext) else 1
                displs = [d * unit for d in displs]
            if kind == "indexed_block":
                return ("indexed_block", blens[0], displs, child)
            if kind == "hindexed_block":
                return ("hindexed_block", blens[0], displs, child)
            if kind == "indexed":
                return ("indexed", blens, displs, child)
            return ("hindexed", blens, displs, child)
        if kind == "resized":
            lb2 = rng.choice([lb, lb - 8, lb + 4, 0])
            ext2 = rng.choice([ext, ext + 16, span + 8, max(1, span), -span - 4])
            return ("resized", lb2, ext2, child)
        if kind == "subarray":
            nd = rng.randint(1, 3)
            sizes = [rng.randint(1, 5) for _ in range(nd)]
            subs = [rng.randint(1, s) for s in sizes]
            starts = [rng.randint(0, s - sb) for s, sb in zip(sizes, subs)]
            order = rng.choice([yk.SUBARRAY_ORDER_C, yk.SUBARRAY_ORDER_FORTRAN])
            return ("subarray", sizes, subs, starts, order, child)
        # struct of the child and a second field of another shape over the same base type
        other = self.leaf(base) if rng.random() < 0.5 else self.gen(base, max(1, depth - 1))
        s2, (lb2_, ext2_), (tlb2, text2) = self.info(other)
        b1, b2 = rng.randint(1, 3), rng.randint(1, 3)
        d1 = rng.randint(0, 2) * 8
        end1 = d1 + max(ext, text) * b1 + max(0, tlb) + 8
        d2 = end1 + rng.randint(0, 2) * 8 + max(0, -tlb2)
        return ("struct", [b1, b2], [d1, d2], [child, other])

    def free(self):
        for h in reversed(self.keep):
            try:
                self.y.type_free(h)
            except Exception:
                pass
        self.keep = []


def footprint(y, h, count):
    """(lo, hi, size): byte offsets touched by `count` elements relative to the buffer
    pointer.  Taken from the oracle's typemap when `y` is the oracle, because the
    reference's true bounds do not always enclose the typemap (a resized child with a
    negative extent inside a vector, for instance)."""
    import ctypes
    import numpy as np
    size = y.size(h)
    f = getattr(y.lib, "yaksa_oracle_byte_offsets", None)
    if f is not None and size * count > 0:
        out = np.empty(size * count, dtype=np.int64)
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p]
        assert f(h, count, out.ctypes.data) == 0
        return int(out.min()), int(out.max()) + 1, size
    lb, ext = y.extent(h)
    tlb, text = y.true_extent(h)
    lo = tlb + min(0, (count - 1) * ext)
    hi = tlb + text + max(0, (count - 1) * ext)
    return lo, hi, size
