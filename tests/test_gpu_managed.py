"""GPU: packs and unpacks on managed memory (cudaMallocManaged), one of the reference pack
test's memory kinds (test/pack/pack-cuda.c), against the oracle.  The buffers come from
the CUDA runtime through ctypes; the host fills and reads them directly.

Tolerance: byte-identical.
"""
import ctypes
import glob
import os

import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import Pair, assert_same_bytes, fill
from typegen import VALID_OPS, Gen, footprint

pytestmark = pytest.mark.gpu


def cudart():
    cands = ["libcudart.so"]
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        cands += sorted(glob.glob(os.path.join(d, "libcudart.so*")))
    for c in cands:
        try:
            lib = ctypes.CDLL(c)
            lib.cudaMallocManaged.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t, ctypes.c_uint]
            lib.cudaFree.argtypes = [ctypes.c_void_p]
            return lib
        except OSError:
            continue
    pytest.skip("no CUDA runtime library to allocate managed memory with")


class Managed:
    def __init__(self, rt, arr):
        self.rt, self.n = rt, arr.nbytes
        self.p = ctypes.c_void_p()
        assert rt.cudaMallocManaged(ctypes.byref(self.p), max(self.n, 1), 1) == 0
        ctypes.memmove(self.p, arr.ctypes.data, self.n)

    def read(self):
        return np.frombuffer(ctypes.string_at(self.p, self.n), dtype=np.uint8).copy()

    def free(self):
        self.rt.cudaFree(self.p)


@pytest.mark.parametrize("seed", range(3))
def test_managed_buffers_match_oracle(cuda, prod, oracle, seed):
    rt = cudart()
    rng = np.random.default_rng(900 + seed)
    g = Gen(oracle, 14000 + seed, max_depth=3)
    bases = ["int32", "double", "int8", "float", "int64", "c_complex"]
    for i in range(12):
        base = bases[i % len(bases)]
        pair = Pair(prod, oracle, g.gen(base))
        count = int(rng.integers(1, 6))
        lo, hi, size = footprint(oracle, pair.ho, count)
        n = size * count
        op = yk.OP_NAMES[str(rng.choice(VALID_OPS[base]))] if i % 3 == 2 else yk.OP_REPLACE
        typed, packed = fill(rng, hi - lo + 64, base), fill(rng, n + 64, base)
        t_m, p_m = Managed(rt, typed), Managed(rt, packed)
        t_o, p_o = typed.copy(), packed.copy()
        if i % 2 == 0:
            ap = prod.pack(t_m.p.value + 32 - lo, count, pair.hp, 0, p_m.p.value, n, op=op)
            ao = oracle.pack(t_o.ctypes.data + 32 - lo, count, pair.ho, 0, p_o.ctypes.data, n, op=op)
        else:
            ap = prod.unpack(p_m.p.value, n, t_m.p.value + 32 - lo, count, pair.hp, 0, op=op)
            ao = oracle.unpack(p_o.ctypes.data, n, t_o.ctypes.data + 32 - lo, count, pair.ho, 0, op=op)
        cuda.cuda.synchronize()
        assert ap == ao
        assert_same_bytes(p_m.read(), p_o, "managed packed", base)
        assert_same_bytes(t_m.read(), t_o, "managed typed", base)
        t_m.free()
        p_m.free()
        pair.free()
    g.free()
