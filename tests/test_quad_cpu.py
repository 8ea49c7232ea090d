"""Host: the binary128 routines that the GPU's long double operators run (yk_quad.h),
against the C compiler's own _Float128 arithmetic -- libgcc's soft-float, the same code
that computes long double on an aarch64 host, where the oracle and the reference's seq
backend run `*out = *out op *in` in long double.

The inputs are every pair of a list of special values (signed zeros, infinities, quiet
and signalling NaNs with payloads, the subnormal and normal extremes, values next to 1)
and random values drawn so that the hard cases are common: exponents near the overflow
and underflow limits, subnormals, near-cancelling sums, products that round at the
subnormal boundary.  Results must be bit-identical, except that a result which is NaN
on both sides may differ in payload and sign (IEEE 754 leaves NaN propagation open).
Comparisons (the MIN and MAX selects) must match exactly.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "yaksa_gb300", "csrc")

FRAC = (1 << 112) - 1
SIGN = 1 << 127
INF = 0x7FFF << 112
ONE = 0x3FFF << 112


def q(sign, exp, frac):
    return (sign << 127) | (exp << 112) | frac


SPECIALS = [
    0, SIGN, INF, SIGN | INF,
    INF | (1 << 111), SIGN | INF | (1 << 111), INF | (1 << 111) | 0x12345, INF | 1,
    1, SIGN | FRAC, 1 << 112, SIGN | (1 << 112), q(0, 0x7FFE, FRAC), q(1, 0x7FFE, FRAC),
    ONE, SIGN | ONE, ONE | 1, q(0, 0x3FFE, FRAC), q(0, 0x3FFF, 1 << 111), q(0, 0x4000, 1 << 111),
    q(0, 0x3FFE, 0), q(0, 0x7F00, 0x1234), q(0, 0x0100, 0xABCDEF), q(1, 0x3F00, 7),
    q(0, 0x0000, 1 << 111), q(0, 0x3F8F, 0), q(0, 0x4070, 0),
]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not found")
    out = str(tmp_path_factory.mktemp("quad") / "libquad.so")
    subprocess.run([cc, "-std=gnu11", "-O2", "-fPIC", "-shared", "-I", CSRC, "-o", out,
                    os.path.join(HERE, "quad_harness.c")], check=True)
    return ctypes.CDLL(out)


def to_bytes(vals):
    return np.frombuffer(b"".join(int(v).to_bytes(16, "little") for v in vals), dtype=np.uint8)


def from_bytes(buf):
    b = buf.tobytes()
    return [int.from_bytes(b[i:i + 16], "little") for i in range(0, len(b), 16)]


def isnan(v):
    return (v & ~SIGN) > INF


def random_values(rng, n):
    """values with exponents spread over the whole range and crowded at both ends"""
    sign = rng.integers(0, 2, n)
    pick = rng.integers(0, 5, n)
    exp = np.where(pick == 0, rng.integers(0, 0x7FFF, n),
                   np.where(pick == 1, rng.integers(0, 120, n),
                            np.where(pick == 2, rng.integers(0x7FFE - 120, 0x7FFF, n),
                                     np.where(pick == 3, rng.integers(0x3FFF - 200, 0x3FFF + 200, n),
                                              rng.integers(0x2000, 0x6000, n)))))
    hi = rng.integers(0, 1 << 48, n, dtype=np.uint64)
    lo = rng.integers(0, 1 << 63, n, dtype=np.uint64) * 2 + rng.integers(0, 2, n, dtype=np.uint64)
    out = []
    for s, e, h, l, k in zip(sign.tolist(), exp.tolist(), hi.tolist(), lo.tolist(), rng.integers(0, 4, n).tolist()):
        f = (h << 64) | l
        if k == 0:      # short significands: exact and tie cases
            f &= ~((1 << int(rng.integers(60, 112))) - 1)
        out.append(q(s, e, f & FRAC))
    return out


def pairs(rng, n):
    """(a, b) operand lists: all special pairs, random pairs, near-cancelling pairs and
    products that land near the limits of the exponent range"""
    a = [x for x in SPECIALS for _ in SPECIALS]
    b = [y for _ in SPECIALS for y in SPECIALS]
    ra, rb = random_values(rng, n), random_values(rng, n)
    a += ra
    b += rb
    # -a nudged by a few ulps or scaled by one binade: cancellation and alignment shifts
    for x in ra[: n // 2]:
        d = int(rng.integers(-3, 4))
        m = x & ~SIGN
        if m + d <= 0 or ((m + d) >> 112) >= 0x7FFF:
            continue
        y = ((x & SIGN) ^ SIGN) | (m + d)
        a.append(x)
        b.append(y)
    # exponent sums near the subnormal boundary and the overflow threshold
    for _ in range(n // 2):
        ea = int(rng.integers(1, 0x7FFF))
        target = int(rng.choice([int(rng.integers(-120, 8)), int(rng.integers(0x7FF0, 0x8010))]))
        eb = target - ea + 0x3FFF
        if not 0 <= eb < 0x7FFF:
            continue
        fa = int(rng.integers(0, 1 << 62)) << 50 | int(rng.integers(0, 1 << 50))
        fb = int(rng.integers(0, 1 << 62)) << 50 | int(rng.integers(0, 1 << 50))
        a.append(q(int(rng.integers(0, 2)), ea, fa & FRAC))
        b.append(q(int(rng.integers(0, 2)), eb, fb & FRAC))
    return a, b


def run(lib, fn_ours, fn_ref, a, b, width, *lead):
    n = len(a) * 16 // width
    ab, bb = to_bytes(a), to_bytes(b)
    o1, o2 = np.zeros_like(ab), np.zeros_like(ab)
    args = [ab.ctypes.data_as(ctypes.c_void_p), bb.ctypes.data_as(ctypes.c_void_p)]
    getattr(lib, fn_ours)(*lead, *args, o1.ctypes.data_as(ctypes.c_void_p), ctypes.c_long(n))
    getattr(lib, fn_ref)(*lead, *args, o2.ctypes.data_as(ctypes.c_void_p), ctypes.c_long(n))
    return from_bytes(o1), from_bytes(o2)


def check(ours, ref, a, b, what):
    bad = [i for i, (x, y) in enumerate(zip(ours, ref)) if x != y and not (isnan(x) and isnan(y))]
    nan_mismatch = [i for i, (x, y) in enumerate(zip(ours, ref)) if isnan(x) != isnan(y)]
    assert not bad and not nan_mismatch, (
        f"{what}: {len(bad)} differ; first: " +
        "; ".join(f"{a[i]:#034x} , {b[i]:#034x} -> ours {ours[i]:#034x} gcc {ref[i]:#034x}"
                  for i in bad[:4]))


@pytest.mark.parametrize("op,name", [(0, "add"), (1, "mul"), (2, "sub"), (3, "lt")])
def test_binary128_against_gcc(lib, op, name):
    rng = np.random.default_rng(1000 + op)
    a, b = pairs(rng, 40000)
    ours, ref = run(lib, "quad_ours", "quad_gcc", a, b, 16, ctypes.c_int(op))
    check(ours, ref, a, b, name)


def test_binary128_complex_mul_against_gcc(lib):
    """Annex G complex multiplication: every (re, im) pair of a short component list,
    times every other, plus random complex values"""
    rng = np.random.default_rng(77)
    comps = [0, SIGN, INF, SIGN | INF, INF | (1 << 111), SIGN | INF | (1 << 111), ONE, SIGN | ONE,
             q(0, 0x7FF0, 5), q(0, 0x0010, 3), q(0, 0x4000, 1 << 110)]
    elems = [(r, i) for r in comps for i in comps]
    ra = random_values(rng, 8000)
    elems_r = list(zip(ra[0::2], ra[1::2]))
    a, b = [], []
    for x in elems:
        for y in elems:
            a += list(x)
            b += list(y)
    for k in range(len(elems_r) - 1):
        a += list(elems_r[k])
        b += list(elems_r[k + 1])
    ours, ref = run(lib, "cquad_ours", "cquad_gcc", a, b, 32)
    check(ours, ref, a, b, "cmul")
