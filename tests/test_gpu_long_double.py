"""GPU: long double and long double complex operators (binary128), against the oracle.

The reference's seq backend applies SUM, PROD, MIN and MAX to long double and SUM and
PROD to long double complex (src/backend/gencomm.py:14-27), computing `*out = *out op
*in` in the host's long double.  On an aarch64 host that is IEEE binary128, which the
GPU computes in integer registers (yaksa_gb300/csrc/yk_quad.h); the oracle computes
with the host compiler, so the two sides are independent implementations.  The tests
run where the host's long double is binary128 and are skipped elsewhere (on x86_64 the
library refuses these operators, see test_gpu_failures.py).

Inputs: every pair of a list of special values (signed zeros, infinities, quiet and
signalling NaNs with payloads, subnormal and normal extremes, values next to 1), every
(re, im) pair of a shorter component list for the complex type plus the Annex G cases,
and random values with exponents across the whole range.  Each runs through the kernel
families that take operators: the runtime-operator typed kernel (contiguous and strided
targets), the sorted-block owner kernel (overlapping indexed_block targets) and the
ordered warp kernel (overlapping targets in no order).  REPLACE into overlapping long
double targets and the long double + int pair type are covered too.

Tolerance: bit-identical, except that an arithmetic result (SUM, PROD) that is NaN on
both sides may differ in NaN payload and sign; every NaN must sit at the same position,
and MIN/MAX (selects) must match NaN payloads too.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import dev_copy

BINARY128 = np.finfo(np.longdouble).nmant == 112
pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not BINARY128, reason="the host's long double is not binary128")]

SIGN = 1 << 127
INF = 0x7FFF << 112
FRAC = (1 << 112) - 1
ONE = 0x3FFF << 112


def q(s, e, f):
    return (s << 127) | (e << 112) | f


LD = [0, SIGN, INF, SIGN | INF, INF | (1 << 111), SIGN | INF | (1 << 111), INF | (1 << 111) | 0x12345,
      INF | 1, 1, SIGN | FRAC, 1 << 112, SIGN | (1 << 112), q(0, 0x7FFE, FRAC), q(1, 0x7FFE, FRAC),
      ONE, SIGN | ONE, ONE | 1, q(0, 0x3FFE, FRAC), q(0, 0x4000, 1 << 111), q(0, 0x3FFE, 0),
      q(0, 0x7F00, 0x1234), q(0, 0x0100, 0xABCDEF), q(0, 0, 1 << 111), q(1, 0x3F00, 7)]
CLD = [0, SIGN, INF, SIGN | INF, INF | (1 << 111), SIGN | INF | (1 << 111), ONE, SIGN | ONE,
       q(0, 0x7FF0, 5), q(0, 0x0010, 3), q(0, 0x4000, 1 << 110)]


def to_bytes(vals):
    """16 little-endian bytes per value"""
    v = np.array([[x & ((1 << 64) - 1), x >> 64] for x in vals], dtype=np.uint64)
    return v.view(np.uint8).ravel()


def words(buf):
    """(n, 2) uint64 view: low and high halves of each 16-byte component"""
    return buf.view(np.uint64).reshape(-1, 2)


def isnan(w):
    return ((w[:, 1] & np.uint64((1 << 63) - 1)) > np.uint64(0x7FFF << 48)) | \
        (((w[:, 1] & np.uint64((1 << 63) - 1)) == np.uint64(0x7FFF << 48)) & (w[:, 0] != 0))


def assert_q_equal(got, exp, op, what):
    g, e = words(got), words(exp)
    diff = (g != e).any(axis=1)
    if op in ("SUM", "PROD"):
        diff &= ~(isnan(g) & isnan(e))
    if diff.any():
        k = np.nonzero(diff)[0][:4]
        fmt = lambda w: [f"{int(h):016x}{int(l):016x}" for l, h in w[k]]
        raise AssertionError(f"{what} {op}: {int(diff.sum())} components differ, first at {k.tolist()}: "
                             f"gpu {fmt(g)} vs oracle {fmt(e)}")
    assert (isnan(g) == isnan(e)).all()


def random_q(rng, n):
    """random binary128 bit patterns, exponents across the range and crowded at both ends"""
    s = rng.integers(0, 2, n).astype(np.uint64)
    pick = rng.integers(0, 4, n)
    e = np.where(pick == 0, rng.integers(0, 0x7FFF, n),
                 np.where(pick == 1, rng.integers(0, 200, n),
                          np.where(pick == 2, rng.integers(0x7FFE - 200, 0x7FFF, n),
                                   rng.integers(0x3FFF - 300, 0x3FFF + 300, n)))).astype(np.uint64)
    hi = (s << np.uint64(63)) | (e << np.uint64(48)) | rng.integers(0, 1 << 48, n, dtype=np.uint64)
    lo = rng.integers(0, 1 << 63, n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n, dtype=np.uint64)
    return np.stack([lo, hi], axis=1).view(np.uint8).ravel()


def run_both(cuda, prod, oracle, tp, to, count, direction, op, typed0, packed0):
    opc = getattr(yk, "OP_" + op)
    t_d, p_d = dev_copy(cuda, typed0), dev_copy(cuda, packed0)
    t_h, p_h = typed0.copy(), packed0.copy()
    n = packed0.nbytes
    if direction == "unpack":
        a = prod.unpack(p_d.data_ptr(), n, t_d.data_ptr(), count, tp, 0, op=opc)
        b = oracle.unpack(p_h.ctypes.data, n, t_h.ctypes.data, count, to, 0, op=opc)
    else:
        a = prod.pack(t_d.data_ptr(), count, tp, 0, p_d.data_ptr(), n, op=opc)
        b = oracle.pack(t_h.ctypes.data, count, to, 0, p_h.ctypes.data, n, op=opc)
    cuda.cuda.synchronize()
    assert a == b == n
    return (t_d.cpu().numpy(), p_d.cpu().numpy()), (t_h, p_h)


def every_pair(vals):
    m = len(vals)
    return [vals[i] for i in range(m) for _ in range(m)], [vals[j] for _ in range(m) for j in range(m)]


def complex_pairs():
    elems = [(r, i) for r in CLD for i in CLD]
    ins, outs = [], []
    for x in elems:
        for y in elems:
            ins += list(x)
            outs += list(y)
    huge = q(0, 0x7FF0, 1)
    nan = INF | (1 << 111)
    annex_g = [((INF, nan), (ONE, ONE)), ((nan, INF), (ONE, SIGN | ONE)), ((ONE, ONE), (INF, nan)),
               ((nan, huge), (huge, huge)), ((huge, nan), (huge, SIGN | huge)), ((0, 0), (INF, INF)),
               ((INF, INF), (0, 0)), ((SIGN | INF, nan), (nan, ONE)), ((nan, nan), (INF, ONE)),
               ((huge, huge), (nan, huge))]
    for a, b in annex_g:
        ins += list(a)
        outs += list(b)
    return ins, outs


@pytest.mark.parametrize("op", ["SUM", "PROD", "MIN", "MAX"])
@pytest.mark.parametrize("direction", ["unpack", "pack"])
def test_long_double_every_pair(cuda, prod, oracle, op, direction):
    """target = op(target, in) over every pair of special values (typed kernel)"""
    ins, outs = every_pair(LD)
    n = len(ins)
    tp, to = prod.type_create_contig(n, yk.TYPE_LONG_DOUBLE), oracle.type_create_contig(n, yk.TYPE_LONG_DOUBLE)
    if direction == "unpack":
        typed0, packed0 = to_bytes(outs), to_bytes(ins)
    else:
        typed0, packed0 = to_bytes(ins), to_bytes(outs)
    (tg, pg), (th, ph) = run_both(cuda, prod, oracle, tp, to, 1, direction, op, typed0, packed0)
    assert_q_equal(tg, th, op, "typed")
    assert_q_equal(pg, ph, op, "packed")
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("op", ["SUM", "PROD"])
def test_long_double_complex_every_pair(cuda, prod, oracle, op):
    """long double complex: every (re, im) pair of the component list times every other,
    and the Annex G cases whose naive product is NaN in both parts"""
    ins, outs = complex_pairs()
    n = len(ins) // 2
    h = yk.TYPE_C_LONG_DOUBLE_COMPLEX
    tp, to = prod.type_create_contig(n, h), oracle.type_create_contig(n, h)
    (tg, _), (th, _) = run_both(cuda, prod, oracle, tp, to, 1, "unpack", op, to_bytes(outs), to_bytes(ins))
    assert_q_equal(tg, th, op, "typed")
    prod.type_free(tp)
    oracle.type_free(to)


CASES = [(yk.TYPE_LONG_DOUBLE, o) for o in ("SUM", "PROD", "MIN", "MAX", "REPLACE")] + \
    [(yk.TYPE_C_LONG_DOUBLE_COMPLEX, o) for o in ("SUM", "PROD", "REPLACE")]


def elem_bytes(h):
    return 16 if h == yk.TYPE_LONG_DOUBLE else 32


@pytest.mark.parametrize("h,op", CASES)
def test_sorted_overlapping_blocks(cuda, prod, oracle, h, op):
    """indexed_block of 6-element blocks at sorted random offsets that overlap (the
    sorted-block owner kernel folds each target element's contributions in block order)"""
    rng = np.random.default_rng(5)
    es = elem_bytes(h)
    nel, nb = 2000, 700
    offs = np.sort(rng.integers(0, nel - 6, nb)).tolist()
    tp, to = prod.type_create_indexed_block(6, offs, h), oracle.type_create_indexed_block(6, offs, h)
    specials = to_bytes(LD).reshape(-1, 16)
    typed0 = specials[rng.integers(0, len(LD), nel * es // 16)].ravel()
    packed0 = np.concatenate([random_q(rng, nb * 6 * es // 32), specials[rng.integers(0, len(LD), nb * 6 * es // 32)].ravel()])
    (tg, _), (th, _) = run_both(cuda, prod, oracle, tp, to, 1, "unpack", op, typed0, packed0)
    assert_q_equal(tg, th, op, "typed")
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("h,op", CASES)
def test_unsorted_overlap(cuda, prod, oracle, h, op):
    """indexed targets that overlap in no order: the ordered warp kernel applies the
    contributions in packed order"""
    rng = np.random.default_rng(9)
    es = elem_bytes(h)
    nel = 300
    blens = rng.integers(1, 5, 120).tolist()
    displs = rng.integers(0, nel - 5, 120).tolist()
    tp, to = prod.type_create_indexed(blens, displs, h), oracle.type_create_indexed(blens, displs, h)
    n = sum(blens) * es
    typed0 = random_q(rng, nel * es // 16)
    packed0 = random_q(rng, n // 16)
    (tg, _), (th, _) = run_both(cuda, prod, oracle, tp, to, 1, "unpack", op, typed0, packed0)
    assert_q_equal(tg, th, op, "typed")
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("h,op", CASES)
@pytest.mark.parametrize("direction", ["unpack", "pack"])
def test_strided_random(cuda, prod, oracle, h, op, direction):
    """hvector of 3-element blocks at a stride of 5 elements, count 3, random values
    across the exponent range (about 96k operations)"""
    rng = np.random.default_rng(11)
    es = elem_bytes(h)
    nblk = 32768 // (es // 16)
    tp, to = prod.type_create_hvector(nblk, 3, 5 * es, h), oracle.type_create_hvector(nblk, 3, 5 * es, h)
    ext = prod.extent(tp)[1]
    typed0 = random_q(rng, 3 * ext // 16)
    packed0 = random_q(rng, 3 * nblk * 3 * es // 16)
    (tg, pg), (th, ph) = run_both(cuda, prod, oracle, tp, to, 3, direction, op, typed0, packed0)
    assert_q_equal(tg, th, op, "typed")
    assert_q_equal(pg, ph, op, "packed")
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("op", ["SUM", "PROD", "MIN", "MAX"])
def test_long_double_int_pair(cuda, prod, oracle, op):
    """the long double + int pair type: the operator applies field by field"""
    rng = np.random.default_rng(3)
    h = yk.TYPE_LONG_DOUBLE_INT
    n = 5000
    size = prod.size(h)
    tp, to = prod.type_create_contig(n, h), oracle.type_create_contig(n, h)
    ext = prod.extent(tp)[1]
    typed0 = random_q(rng, ext // 16)
    packed0 = random_q(rng, n * size // 16)[: n * size]
    (tg, _), (th, _) = run_both(cuda, prod, oracle, tp, to, 1, "unpack", op, typed0, packed0)
    if op in ("MIN", "MAX"):
        assert np.array_equal(tg, th)
    else:
        # compare the long double fields with the NaN exemption, the rest exactly
        ld = np.zeros(len(tg), dtype=bool)
        for i in range(n):
            ld[i * ext // n: i * ext // n + 16] = True
        assert_q_equal(tg[ld], th[ld], op, "long double fields")
        assert np.array_equal(tg[~ld], th[~ld])
    prod.type_free(tp)
    oracle.type_free(to)


def test_server_refuses_long_double_arithmetic(cuda, prod):
    """the persistent server has no binary128 operators: it refuses them at submission
    and still takes REPLACE of the same type"""
    t = prod.type_create_contig(4, yk.TYPE_LONG_DOUBLE)
    buf = cuda.zeros(256, dtype=cuda.uint8, device="cuda")
    srv = yk.Server(prod, ring_requests=8)
    try:
        with pytest.raises(yk.YaksaError) as e:
            srv.submit(yk.unpack_op(buf.data_ptr(), 64, buf.data_ptr() + 64, 1, t, 0, op=yk.OP_SUM))
        assert e.value.rc == yk.ERR_NOT_SUPPORTED
        tk = srv.submit(yk.unpack_op(buf.data_ptr(), 64, buf.data_ptr() + 128, 1, t, 0))
        srv.wait(tk)
    finally:
        srv.destroy()
        prod.type_free(t)
