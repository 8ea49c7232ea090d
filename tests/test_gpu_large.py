"""GPU: packed ranges beyond 4 GiB, which take the kernels' 64-bit position arithmetic
(the halo and reduction configs stay below it).  Checked by properties that do not need
the oracle at this size: the packed bytes equal a strided torch view of the typed
buffer, unpack restores exactly the typed bytes the type covers, a float SUM unpack
equals torch's own IEEE round-to-nearest additions, and every hindexed block lands
where its displacement says.

Tolerance: byte-identical (float SUM of one addend per element rounds identically on
both sides).  About 20 GB of device memory per test.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk

pytestmark = pytest.mark.gpu

N = (1 << 29) + 12345        # elements of 2 floats: 4.3 GB packed


def test_hvector_roundtrip_beyond_4gib(cuda, prod):
    t = prod.type_create_hvector(N, 2, 12, yk.TYPE_FLOAT)      # 2 of every 3 floats
    assert prod.size(t) == N * 8 and N * 8 > (1 << 32)
    g = cuda.Generator(device="cuda").manual_seed(5)
    src = cuda.rand(N * 3, device="cuda", generator=g)
    packed = cuda.empty(N * 2, device="cuda")
    assert prod.pack(src.data_ptr(), 1, t, 0, packed.data_ptr(), N * 8) == N * 8
    cuda.cuda.synchronize()
    assert cuda.equal(packed.view(N, 2), src.view(N, 3)[:, :2])
    dst = cuda.zeros(N * 3, device="cuda")
    assert prod.unpack(packed.data_ptr(), N * 8, dst.data_ptr(), 1, t, 0) == N * 8
    cuda.cuda.synchronize()
    assert cuda.equal(dst.view(N, 3)[:, :2], src.view(N, 3)[:, :2])
    assert int((dst.view(N, 3)[:, 2] != 0).sum()) == 0
    # a partial range across the 2^32 boundary, and one past the end (clipped)
    a, n = (1 << 32) - (1 << 19), (1 << 19) + (1 << 16)   # the range ends at 2^32 + 98,760
    assert a + n < N * 8
    out = cuda.zeros(n // 4, device="cuda")
    assert prod.pack(src.data_ptr(), 1, t, a, out.data_ptr(), n) == n
    cuda.cuda.synchronize()
    assert cuda.equal(out, packed.view(-1)[a // 4:(a + n) // 4])
    a = (1 << 32) + 4096
    assert prod.pack(src.data_ptr(), 1, t, a, out.data_ptr(), n) == N * 8 - a
    cuda.cuda.synchronize()
    assert cuda.equal(out[:(N * 8 - a) // 4], packed.view(-1)[a // 4:])
    prod.type_free(t)


def test_sum_unpack_beyond_4gib(cuda, prod):
    t = prod.type_create_hvector(N, 2, 12, yk.TYPE_FLOAT)
    g = cuda.Generator(device="cuda").manual_seed(6)
    target = cuda.rand(N * 3, device="cuda", generator=g) * 2 - 1
    packed = cuda.rand(N * 2, device="cuda", generator=g) * 2 - 1
    expect = target.clone()
    expect.view(N, 3)[:, :2] += packed.view(N, 2)
    assert prod.unpack(packed.data_ptr(), N * 8, target.data_ptr(), 1, t, 0, op=yk.OP_SUM) == N * 8
    cuda.cuda.synchronize()
    assert cuda.equal(target, expect)
    prod.type_free(t)


def test_hindexed_beyond_4gib(cuda, prod):
    rng = np.random.default_rng(7)
    nb = 1024
    blens = rng.integers(1 << 20, (1 << 20) + (1 << 18), nb).astype(np.int64)   # int32 elements
    assert int(blens.sum()) * 4 > (1 << 32)
    gaps = rng.integers(0, 4096, nb)
    order = rng.permutation(nb)
    starts = np.cumsum(blens[order] + gaps) - blens[order]
    displs = np.empty(nb, dtype=np.int64)
    displs[order] = starts * 4
    span = int(starts[-1] + blens[order][-1])
    t = prod.type_create_hindexed_arrays(nb, blens.ctypes.data, displs.ctypes.data, yk.TYPE_INT32_T)
    total = int(blens.sum())
    typed = cuda.randint(-(1 << 31), (1 << 31) - 1, (span,), dtype=cuda.int32, device="cuda")
    packed = cuda.empty(total, dtype=cuda.int32, device="cuda")
    assert prod.pack(typed.data_ptr(), 1, t, 0, packed.data_ptr(), total * 4) == total * 4
    back = cuda.zeros_like(typed)
    assert prod.unpack(packed.data_ptr(), total * 4, back.data_ptr(), 1, t, 0) == total * 4
    cuda.cuda.synchronize()
    pos = 0
    for j in range(nb):
        d, n = int(displs[j]) // 4, int(blens[j])
        assert cuda.equal(packed[pos:pos + n], typed[d:d + n]), j
        assert cuda.equal(back[d:d + n], typed[d:d + n]), j
        pos += n
    prod.type_free(t)
