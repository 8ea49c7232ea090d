"""Shared helpers for the parity tests: typed buffer filling and one pack/unpack
round on the GPU engine and on the CPU oracle with the same inputs."""
import numpy as np

import yaksa_gb300 as yk
from typegen import BASE, build, footprint


def fill(rng, nbytes, base):
    """nbytes of valid values of `base` (finite floats, 0/1 bools, any integer bits)."""
    dt = BASE[base][2] if base in BASE else None
    out = np.empty(nbytes, dtype=np.uint8)
    if dt is None or dt.startswith("i") or dt.startswith("u"):
        out[:] = rng.integers(0, 256, nbytes, dtype=np.uint8)
    elif dt == "bool":
        out[:] = rng.integers(0, 2, nbytes, dtype=np.uint8)
    else:
        comp = np.float32 if dt in ("f4", "c8") else np.float64
        n = nbytes // np.dtype(comp).itemsize
        vals = rng.uniform(-1.0, 1.0, n).astype(comp)
        out[:n * np.dtype(comp).itemsize] = vals.view(np.uint8)
        out[n * np.dtype(comp).itemsize:] = 0
    return out


class Pair:
    """The same recipe instantiated on the GPU engine and the oracle."""

    def __init__(self, prod, oracle, recipe):
        self.prod, self.oracle = prod, oracle
        self.keep_p, self.keep_o = [], []
        self.hp = build(prod, recipe, self.keep_p)
        self.ho = build(oracle, recipe, self.keep_o)

    def free(self):
        for y, keep in ((self.prod, self.keep_p), (self.oracle, self.keep_o)):
            for h in reversed(keep):
                y.type_free(h)


def dev_copy(torch, arr):
    t = torch.empty(arr.nbytes, dtype=torch.uint8, device="cuda")
    t.copy_(torch.from_numpy(arr))
    # the engine runs on its own streams: make the copy complete device-wide
    torch.cuda.synchronize()
    return t


def host_of(torch, t):
    return t.cpu().numpy()


def segments(rng, total, unit, nseg):
    """Split [0, total) into nseg pieces whose starts fall on multiples of `unit`."""
    if nseg <= 1 or total <= unit:
        return [(0, total)]
    cuts = sorted(set(int(c) * unit for c in rng.integers(1, max(2, total // unit), nseg - 1)))
    starts = [0] + [c for c in cuts if 0 < c < total]
    out = []
    for i, s in enumerate(starts):
        e = starts[i + 1] if i + 1 < len(starts) else total
        out.append((s, e - s))
    return out


def roundtrip(torch, pair, count, base, op, rng, nseg=1, direction="both", ragged=False):
    """Pack (typed -> packed) then unpack (packed -> typed) on both libraries; returns
    the four result buffers (packed_gpu, packed_cpu, typed_gpu, typed_cpu) and the
    actual byte counts of every call."""
    prod, oracle = pair.prod, pair.oracle
    lo, hi, size = footprint(oracle, pair.ho, count)
    total = size * count
    pad = 64
    typed = fill(rng, hi - lo + 2 * pad, base)
    packed0 = fill(rng, total + pad, base)
    dst0 = fill(rng, hi - lo + 2 * pad, base)

    # oracle (host buffers)
    t_o, p_o, d_o = typed.copy(), packed0.copy(), dst0.copy()
    t_p, p_p, d_p = dev_copy(torch, typed), dev_copy(torch, packed0), dev_copy(torch, dst0)
    opc = yk.OP_NAMES[op]
    unit = 1
    bsz = BASE[base][1] if base in BASE else 1
    unit = bsz
    segs = segments(rng, total, unit, nseg)
    actual = []
    for (s, n) in segs:
        ask = n + (rng.integers(0, unit) if ragged else 0)
        if direction in ("both", "pack"):
            ao = oracle.pack(t_o.ctypes.data + pad - lo, count, pair.ho, s, p_o.ctypes.data + s, ask,
                             op=opc if direction == "pack" else yk.OP_REPLACE)
            ap = prod.pack(t_p.data_ptr() + pad - lo, count, pair.hp, s, p_p.data_ptr() + s, ask,
                           op=opc if direction == "pack" else yk.OP_REPLACE)
            actual.append(("pack", s, ao, ap))
    if direction == "unpack":
        # unpack from the initial packed buffer
        pass
    for (s, n) in segs:
        if direction in ("both", "unpack"):
            ao = oracle.unpack(p_o.ctypes.data + s, n, d_o.ctypes.data + pad - lo, count, pair.ho, s,
                               op=opc)
            ap = prod.unpack(p_p.data_ptr() + s, n, d_p.data_ptr() + pad - lo, count, pair.hp, s,
                             op=opc)
            actual.append(("unpack", s, ao, ap))
    torch.cuda.synchronize()
    return (host_of(torch, p_p), p_o, host_of(torch, d_p), d_o, actual)


def assert_same_bytes(a, b, what, base=None):
    if np.array_equal(a, b):
        return
    bad = np.nonzero(a != b)[0]
    # float NaN payloads are not pinned: accept NaN-vs-NaN at the same element
    if base in ("float", "double", "c_complex", "c_double_complex"):
        comp = np.float32 if base in ("float", "c_complex") else np.float64
        w = np.dtype(comp).itemsize
        n = len(a) // w
        av, bv = a[:n * w].view(comp), b[:n * w].view(comp)
        neq = ~((av == bv) | (np.isnan(av) & np.isnan(bv)))
        if not neq.any() and np.array_equal(a[n * w:], b[n * w:]):
            return
    raise AssertionError(f"{what}: {len(bad)} bytes differ, first at {bad[:8].tolist()}: "
                         f"gpu {a[bad[:8]].tolist()} vs oracle {b[bad[:8]].tolist()}")
