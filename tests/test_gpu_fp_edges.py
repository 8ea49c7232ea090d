"""GPU: floating-point operators at the edges of IEEE arithmetic, against the oracle.

The inputs are every pair of a list of special values: +-0, +-inf, quiet NaNs with
payloads and both signs, a signalling NaN, the smallest and largest subnormals, the
smallest and largest normals (so sums and products overflow to infinity and underflow
to subnormals or zero), +-1 and a few ordinary values.  Complex values take every pair
of a shorter list as (real, imaginary), and include the inputs that make the naive
product (ac - bd) + i(ad + bc) NaN in both parts, so the infinity recovery of ISO C
Annex G.5.1 runs: (inf + NaN i)(1 + i), (NaN + 1e30 i)(1e30 + 1e30 i) and so on.  The
oracle computes with the host compiler's own arithmetic, as the reference's seq backend
does (`*out *= *in` on _Complex values calls libgcc's __mulsc3/__muldc3 on that path).

Each (base type, operator) runs through three kernel families: the runtime-operator
typed kernel (contiguous target), the compile-time-operator sorted-block kernels
(indexed_block targets whose blocks overlap, folded in block order), and a strided
hvector target.  Pack with an operator (packed = op(typed, packed)) is covered on the
contiguous layout.

Tolerance: bit-identical, with one exception that the test confines exactly: an
arithmetic result (SUM, PROD) that is NaN on both sides may differ in NaN payload and
sign, because the GPU returns the canonical NaN where the host propagates an input's
payload.  Every NaN must sit at the same position on both sides, and MIN/MAX, which
select one input bit for bit, must match NaN payloads too.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import dev_copy

pytestmark = pytest.mark.gpu

F32 = [0x00000000, 0x80000000, 0x7f800000, 0xff800000, 0x7fc00000, 0xffc00000, 0x7fc12345,
       0x7f800001, 0x00000001, 0x807fffff, 0x00800000, 0x80800000, 0x7f7fffff, 0xff7fffff,
       0x3f800000, 0xbf800000, 0x60ad78ec, 0x1e3ce508, 0x40400000, 0x3f000000]
F64 = [0x0000000000000000, 0x8000000000000000, 0x7ff0000000000000, 0xfff0000000000000,
       0x7ff8000000000000, 0xfff8000000000000, 0x7ff8000000012345, 0x7ff0000000000001,
       0x0000000000000001, 0x800fffffffffffff, 0x0010000000000000, 0x8010000000000000,
       0x7fefffffffffffff, 0xffefffffffffffff, 0x3ff0000000000000, 0xbff0000000000000,
       0x7e37e43c8800759c, 0x01a56e1fc2f8f359, 0x4008000000000000, 0x3fe0000000000000]
# components of complex values: 0, -0, inf, -inf, NaN, -NaN, 1, -1, huge, tiny, 2.5
C32 = [0x00000000, 0x80000000, 0x7f800000, 0xff800000, 0x7fc00000, 0xffc00000, 0x3f800000,
       0xbf800000, 0x7149f2ca, 0x0da24260, 0x40200000]
C64 = [0x0000000000000000, 0x8000000000000000, 0x7ff0000000000000, 0xfff0000000000000,
       0x7ff8000000000000, 0xfff8000000000000, 0x3ff0000000000000, 0xbff0000000000000,
       0x7e37e43c8800759c, 0x01a56e1fc2f8f359, 0x4004000000000000]

# base name -> (type handle, component dtype, bit dtype, components per element, specials)
BASES = {"float": (yk.TYPE_FLOAT, np.float32, np.uint32, 1, F32),
         "double": (yk.TYPE_DOUBLE, np.float64, np.uint64, 1, F64),
         "c_complex": (yk.TYPE_C_COMPLEX, np.float32, np.uint32, 2, C32),
         "c_double_complex": (yk.TYPE_C_DOUBLE_COMPLEX, np.float64, np.uint64, 2, C64)}
OPS = {"float": ("SUM", "PROD", "MIN", "MAX"), "double": ("SUM", "PROD", "MIN", "MAX"),
       "c_complex": ("SUM", "PROD"), "c_double_complex": ("SUM", "PROD")}


def elements(base):
    """Every special value (real) or every (re, im) pair of special components, as bits."""
    _, _, bt, nc, sp = BASES[base]
    sp = np.array(sp, dtype=bt)
    if nc == 1:
        return sp.reshape(-1, 1)
    re, im = np.meshgrid(sp, sp, indexing="ij")
    return np.stack([re.ravel(), im.ravel()], axis=1)


def annex_g_cases(base):
    """(in, out) complex pairs whose naive product is NaN in both parts."""
    _, comp, bt, _, _ = BASES[base]
    inf, nan = comp(np.inf), comp(np.nan)
    huge = comp(1e30) if comp is np.float32 else comp(1e300)
    pairs = [((inf, nan), (1, 1)), ((nan, inf), (2, -3)), ((1, 1), (inf, nan)),
             ((nan, huge), (huge, huge)), ((huge, nan), (huge, -huge)), ((0, 0), (inf, inf)),
             ((inf, inf), (0, 0)), ((-inf, nan), (nan, 2)), ((nan, nan), (inf, 1)),
             ((huge, huge), (nan, huge))]
    ins = np.array([[comp(a), comp(b)] for (a, b), _ in pairs], dtype=comp).view(bt)
    outs = np.array([[comp(c), comp(d)] for _, (c, d) in pairs], dtype=comp).view(bt)
    return ins, outs


def all_pairs(base):
    """(in, out) element arrays (bits, shape (n, components)) covering every pair."""
    e = elements(base)
    m = len(e)
    ins, outs = e[np.repeat(np.arange(m), m)], e[np.tile(np.arange(m), m)]
    if BASES[base][3] == 2:
        gi, go = annex_g_cases(base)
        ins, outs = np.concatenate([ins, gi]), np.concatenate([outs, go])
    return ins, outs


def assert_fp_equal(got, exp, base, op, what):
    """Bit-identical, except NaN payload/sign of arithmetic results NaN on both sides."""
    _, comp, bt, _, _ = BASES[base]
    g, e = got.view(bt), exp.view(bt)
    gf, ef = got.view(comp), exp.view(comp)
    diff = g != e
    if op in ("SUM", "PROD"):
        diff &= ~(np.isnan(gf) & np.isnan(ef))
    if diff.any():
        k = np.nonzero(diff)[0][:6]
        raise AssertionError(f"{what} {base} {op}: {int(diff.sum())} components differ, first at "
                             f"{k.tolist()}: gpu {[hex(int(x)) for x in g[k]]} vs oracle "
                             f"{[hex(int(x)) for x in e[k]]}")
    assert (np.isnan(gf) == np.isnan(ef)).all()


def run_both(cuda, prod, oracle, tp, to, count, direction, op, typed0, packed0, lo=0):
    """One unpack (or pack) with `op` on the GPU and on the oracle from the same bytes;
    returns ((typed_gpu, packed_gpu), (typed_cpu, packed_cpu))."""
    opc = getattr(yk, "OP_" + op)
    t_d, p_d = dev_copy(cuda, typed0), dev_copy(cuda, packed0)
    t_h, p_h = typed0.copy(), packed0.copy()
    n = packed0.nbytes
    if direction == "unpack":
        a = prod.unpack(p_d.data_ptr(), n, t_d.data_ptr() - lo, count, tp, 0, op=opc)
        b = oracle.unpack(p_h.ctypes.data, n, t_h.ctypes.data - lo, count, to, 0, op=opc)
    else:
        a = prod.pack(t_d.data_ptr() - lo, count, tp, 0, p_d.data_ptr(), n, op=opc)
        b = oracle.pack(t_h.ctypes.data - lo, count, to, 0, p_h.ctypes.data, n, op=opc)
    cuda.cuda.synchronize()
    assert a == b
    return (t_d.cpu().numpy(), p_d.cpu().numpy()), (t_h, p_h)


CASES = [(b, o) for b in BASES for o in OPS[b]]


@pytest.mark.parametrize("base,op", CASES)
@pytest.mark.parametrize("direction", ["unpack", "pack"])
def test_contiguous_every_pair(cuda, prod, oracle, base, op, direction):
    """target[i] = op(in[i], target[i]) over every pair of special values (typed kernel)."""
    h, comp, bt, nc, _ = BASES[base]
    ins, outs = all_pairs(base)
    n = len(ins)
    tp, to = prod.type_create_contig(n, h), oracle.type_create_contig(n, h)
    # unpack: packed holds `in`, the target `out`; pack: the typed buffer is `in`
    if direction == "unpack":
        typed0, packed0 = outs.astype(bt).view(np.uint8).ravel(), ins.astype(bt).view(np.uint8).ravel()
    else:
        typed0, packed0 = ins.astype(bt).view(np.uint8).ravel(), outs.astype(bt).view(np.uint8).ravel()
    (tg, pg), (th, ph) = run_both(cuda, prod, oracle, tp, to, 1, direction, op, typed0, packed0)
    assert_fp_equal(tg.view(comp), th.view(comp), base, op, "typed")
    assert_fp_equal(pg.view(comp), ph.view(comp), base, op, "packed")
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("base,op", CASES)
def test_sorted_overlapping_blocks(cuda, prod, oracle, base, op):
    """indexed_block of 8-element blocks at sorted random offsets that overlap, so most
    target elements fold several special values in block order (the sorted-block lane
    and chunk kernels, compile-time operators)."""
    h, comp, bt, nc, _ = BASES[base]
    rng = np.random.default_rng(17)
    e = elements(base)
    nel, nb = 3000, 1200
    offs = np.sort(rng.integers(0, nel - 8, nb)).tolist()
    tp, to = prod.type_create_indexed_block(8, offs, h), oracle.type_create_indexed_block(8, offs, h)
    typed0 = e[rng.integers(0, len(e), nel)].astype(bt).view(np.uint8).ravel()
    packed0 = e[rng.integers(0, len(e), nb * 8)].astype(bt).view(np.uint8).ravel()
    (tg, pg), (th, ph) = run_both(cuda, prod, oracle, tp, to, 1, "unpack", op, typed0, packed0)
    assert_fp_equal(tg.view(comp), th.view(comp), base, op, "typed")
    prod.type_free(tp)
    oracle.type_free(to)


@pytest.mark.parametrize("base,op", CASES)
def test_strided_hvector(cuda, prod, oracle, base, op):
    """hvector of 3-element blocks at a stride of 5 elements, count 2 of the type."""
    h, comp, bt, nc, _ = BASES[base]
    rng = np.random.default_rng(23)
    e = elements(base)
    es = np.dtype(bt).itemsize * nc
    nblk = 400
    tp = prod.type_create_hvector(nblk, 3, 5 * es, h)
    to = oracle.type_create_hvector(nblk, 3, 5 * es, h)
    ext = prod.extent(tp)[1]
    nel = (ext + ext) // es
    typed0 = e[rng.integers(0, len(e), nel)].astype(bt).view(np.uint8).ravel()
    packed0 = e[rng.integers(0, len(e), 2 * nblk * 3)].astype(bt).view(np.uint8).ravel()
    (tg, pg), (th, ph) = run_both(cuda, prod, oracle, tp, to, 2, "unpack", op, typed0, packed0)
    assert_fp_equal(tg.view(comp), th.view(comp), base, op, "typed")
    prod.type_free(tp)
    oracle.type_free(to)
