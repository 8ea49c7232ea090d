"""GPU: a type rebuilt by yaksa_unflatten from yaksa_flatten's bytes packs and unpacks
like the original (the reference's test/flatten/flatten.c: pack with the type, unpack
with its flattened copy), on seeded random types, against the oracle.

Tolerance: byte-identical (REPLACE only moves bytes).
"""
import numpy as np
import pytest

from helpers import Pair, assert_same_bytes, dev_copy, fill, host_of
from typegen import Gen, footprint

pytestmark = pytest.mark.gpu

BASES = ["int32", "double", "int8", "float", "c_complex", "short_int", "int16", "2int"]


@pytest.mark.parametrize("seed", range(6))
def test_pack_with_type_unpack_with_flattened_copy(cuda, prod, oracle, seed):
    rng = np.random.default_rng(seed)
    g = Gen(oracle, 9000 + seed, max_depth=3)
    for i, base in enumerate(BASES):
        pair = Pair(prod, oracle, g.gen(base))
        u = prod.unflatten(prod.flatten(pair.hp))
        count = int(rng.integers(1, 4))
        lo, hi, size = footprint(oracle, pair.ho, count)
        n = size * count
        typed = fill(rng, hi - lo + 64, base)
        t_g = dev_copy(cuda, typed)
        p_g = cuda.zeros(n + 16, dtype=cuda.uint8, device="cuda")
        assert prod.pack(t_g.data_ptr() + 32 - lo, count, pair.hp, 0, p_g.data_ptr(), n) == n
        d_g = dev_copy(cuda, fill(rng, hi - lo + 64, base))
        d_ref = host_of(cuda, d_g)
        assert prod.unpack(p_g.data_ptr(), n, d_g.data_ptr() + 32 - lo, count, u, 0) == n
        cuda.cuda.synchronize()
        # the oracle: the same round trip with the original type
        po = np.zeros(n + 16, dtype=np.uint8)
        oracle.pack(typed.ctypes.data + 32 - lo, count, pair.ho, 0, po.ctypes.data, n)
        oracle.unpack(po.ctypes.data, n, d_ref.ctypes.data + 32 - lo, count, pair.ho, 0)
        assert_same_bytes(host_of(cuda, p_g), po, f"packed {base}")
        assert_same_bytes(host_of(cuda, d_g), d_ref, f"unpacked {base}")
        prod.type_free(u)
        pair.free()
    g.free()
