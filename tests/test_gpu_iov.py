"""GPU: segment lists written by a kernel (yaksa_gb300_iov_stream) against the host
yaksa_iov of the product (pinned to the reference's own test/iov/iov.c) and of the
oracle: random types of depth <= 3 over every base type including pair builtins, counts
1..5, offsets and length limits that start and stop inside the list.  Entries are
compared as (address, length) pairs, with the same count, and requests the reference
refuses (an offset inside a two-piece pair) are refused too.

Tolerance: exact.
"""
import ctypes

import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import Pair
from typegen import Gen

pytestmark = pytest.mark.gpu


def _device_iov(cuda, prod, buf, count, t, offset, max_len):
    out = cuda.zeros(max(1, max_len) * 16, dtype=cuda.uint8, device="cuda")
    n = ctypes.c_size_t()
    h = ctypes.c_void_p(cuda.cuda.current_stream().cuda_stream)
    lib = prod.lib
    lib.yaksa_gb300_iov_stream.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_size_t,
                                           ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                           ctypes.c_void_p]
    lib.yaksa_gb300_iov_stream.restype = ctypes.c_int
    rc = lib.yaksa_gb300_iov_stream(buf, count, t, offset, out.data_ptr(), max_len, ctypes.byref(n),
                                    ctypes.addressof(h))
    cuda.cuda.synchronize()
    if rc:
        return rc, None
    v = out.cpu().numpy().view(np.uint64)[: 2 * n.value].reshape(-1, 2)
    return 0, [(int(a), int(b)) for a, b in v]


def _host_iov(y, buf, count, t, offset, max_len):
    try:
        return 0, y.iov(buf, count, t, offset, max_len)
    except yk.YaksaError as e:
        return e.rc, None


@pytest.mark.parametrize("seed", range(6))
def test_device_segment_list_matches_host(cuda, prod, oracle, seed):
    g = Gen(oracle, 9100 + seed, max_depth=3)
    rng = np.random.default_rng(seed)
    buf = 1 << 40                       # an address only: nothing is read or written there
    bases = ["int32", "double", "int8", "float", "short_int", "double_int", "float_int", "int16"]
    for base in bases:
        pair = Pair(prod, oracle, g.gen(base))
        for count in (1, 2, 5):
            total = prod.iov_len(count, pair.hp)
            for _ in range(4):
                off = int(rng.integers(0, total + 1))
                mx = int(rng.integers(1, total + 2))
                want = _host_iov(prod, buf, count, pair.hp, off, mx)
                ref = _host_iov(oracle, buf, count, pair.ho, off, mx)
                got = _device_iov(cuda, prod, buf, count, pair.hp, off, mx)
                assert want == ref, (base, count, off, mx)
                assert got == want, (base, count, off, mx, got and got[:4], want[1] and want[1][:4])
        pair.free()
    g.free()


def test_device_segment_list_large_hindexed(cuda, prod):
    """2^18 shuffled blocks: the whole list at once, then a window in the middle"""
    rng = np.random.default_rng(3)
    nb = 1 << 18
    blens = rng.integers(1, 30, nb)
    displs = (np.cumsum(blens + rng.integers(0, 7, nb)) - blens) * 4
    perm = rng.permutation(nb)
    t = prod.type_create_hindexed(blens[perm].tolist(), displs[perm].tolist(), yk.TYPE_INT32_T)
    buf = 1 << 36
    for off, mx in ((0, nb * 2), (nb // 3, 1000)):
        rc, got = _device_iov(cuda, prod, buf, 2, t, off, mx)
        assert rc == 0
        assert got == prod.iov(buf, 2, t, off, mx)
    prod.type_free(t)
