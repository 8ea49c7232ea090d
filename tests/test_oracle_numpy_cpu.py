"""CPU: the oracle's unpack-with-operator on the reduce configs' shapes and value
distributions, against NumPy's unbuffered ufunc.at, an implementation independent of
the oracle's C.

The reference applies an unpack elementwise in block order: for block b and element j
it sets t[off_b + j] = OP(packed[8b + j], t[off_b + j])
(src/backend/seq/genpup.py:119-211, operators :302-327).  ufunc.at(t, idx, vals) with
idx and vals in that same order applies each pair in turn, so repeated targets
accumulate in block order too.  Cases: double SUM (values N(0, 1)), int64 MAX (the full
range), uint32 BXOR and complex float PROD (|z| in [0.9, 1.1]), over indexed_block
types of 8-element blocks at sorted random offsets whose blocks overlap, at 2^14 blocks
instead of the configs' 2^22.  Floating-point results are compared bit for bit: these
inputs are finite and their products stay finite, so no NaN payload is involved.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk

CASES = [("double", yk.TYPE_DOUBLE, np.float64, yk.OP_SUM, np.add),
         ("int64", yk.TYPE_INT64_T, np.int64, yk.OP_MAX, np.maximum),
         ("uint32", yk.TYPE_UINT32_T, np.uint32, yk.OP_BXOR, np.bitwise_xor),
         ("c_complex", yk.TYPE_C_COMPLEX, np.complex64, yk.OP_PROD, np.multiply)]


def values(rng, name, n):
    if name == "double":
        return rng.standard_normal(n)
    if name == "int64":
        return rng.integers(-(1 << 63), (1 << 63) - 1, n, dtype=np.int64)
    if name == "uint32":
        return rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    r = np.exp(rng.uniform(np.log(0.9), np.log(1.1), n))
    a = rng.uniform(0, 2 * np.pi, n)
    return (r * np.exp(1j * a)).astype(np.complex64)


@pytest.mark.parametrize("name,handle,dt,op,uf", CASES, ids=[c[0] for c in CASES])
def test_oracle_reduce_matches_ufunc_at(oracle, name, handle, dt, op, uf):
    rng = np.random.default_rng(17)
    nblk, bl = 1 << 14, 8
    nel = nblk * bl                     # as many target elements as contributions
    offs = np.sort(rng.integers(0, nel - bl, nblk)).astype(np.int64)
    t = oracle.type_create_indexed_block_array(nblk, bl, offs.ctypes.data, handle)
    target = values(rng, name, nel).astype(dt)
    packed = values(rng, name, nblk * bl).astype(dt)
    got = target.copy()
    n = oracle.unpack(packed.ctypes.data, packed.nbytes, got.ctypes.data, 1, t, 0, op=op)
    assert n == packed.nbytes
    exp = target.copy()
    idx = (offs[:, None] + np.arange(bl)[None, :]).reshape(-1)
    uf.at(exp, idx, packed)
    assert np.array_equal(got.view(np.uint8), exp.view(np.uint8)), \
        f"{name}: {int((got != exp).sum())} elements differ"
    oracle.type_free(t)
