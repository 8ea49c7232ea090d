"""GPU: every launch shape of the contiguous-block hindexed kernels against the oracle.

The autotuner chooses among the shuffle-search kernel's shapes (units per lane,
residency, grid cap) and, for unpacks, the bulk-staged form.  The test hook yaksa_gb300_debug_hidx_shape forces each shape in turn,
so every one is compared with the oracle on the same requests, whatever the tuner would
pick: int32 and double blocks in shuffled order with gaps, single-element blocks, a
packed size that is not a multiple of 16, the whole request and parts that start and
end inside blocks, in both directions.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import dev_copy

pytestmark = pytest.mark.gpu

# (variant, units, ctas): the shuffle kernel's shapes with their default grid, the
# default shape at two waves, and the bulk-staged unpack (variant 3)
SHAPES = [(0, 0, 0), (0, 0, 8), (0, 4, 0), (0, 2, 0), (0, 16, 0), (3, 0, 4)]


@pytest.fixture
def shaped(prod):
    yield prod
    assert prod.lib.yaksa_gb300_debug_hidx_shape(-1, 0, 0) == 0


def _hindexed(prod, oracle, rng, nb, maxlen, base, esize):
    blens = rng.integers(1, maxlen, nb)
    blens[: nb // 10] = 1                              # single-element blocks
    if (int(blens.sum()) * esize) % 16 == 0:
        blens[-1] += 1                                  # packed size not a multiple of 16
    displs = (np.cumsum(blens + rng.integers(0, 5, nb)) - blens) * esize
    perm = rng.permutation(nb)
    args = (blens[perm].tolist(), displs[perm].tolist(), base)
    return prod.type_create_hindexed(*args), oracle.type_create_hindexed(*args)


def _bounds(y, t):
    lb, text = y.true_extent(t)
    return lb, lb + text


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("base,esize,maxlen", [(yk.TYPE_INT32_T, 4, 40), (yk.TYPE_DOUBLE, 8, 300),
                                               (yk.TYPE_INT32_T, 4, 3)])
def test_forced_shape_matches_oracle(cuda, shaped, oracle, shape, base, esize, maxlen):
    prod = shaped
    rng = np.random.default_rng(shape[1] + 7 * esize + maxlen)
    tp, to = _hindexed(prod, oracle, rng, 20011, maxlen, base, esize)
    n = prod.size(tp)
    assert n % 16
    lo, hi = _bounds(prod, tp)
    packed = rng.integers(0, 256, n, dtype=np.uint8)
    target = rng.integers(0, 256, hi - lo, dtype=np.uint8)
    pd, td0 = dev_copy(cuda, packed), dev_copy(cuda, target)
    assert prod.lib.yaksa_gb300_debug_hidx_shape(*shape) == 0
    # the whole request; a part from a 16-byte boundary inside a block to an element
    # boundary short of the end; a part on a packed pointer off 16 bytes
    for b0, b1 in ((0, n), (16 * (n // 48), n - esize * 1001), (esize, n)):
        th = target.copy()
        oracle.unpack(packed.ctypes.data + b0, b1 - b0, th.ctypes.data - lo, 1, to, b0)
        td = dev_copy(cuda, target)
        prod.unpack(pd.data_ptr() + b0, b1 - b0, td.data_ptr() - lo, 1, tp, b0)
        ph = np.zeros(b1 - b0, dtype=np.uint8)
        oracle.pack(target.ctypes.data - lo, 1, to, b0, ph.ctypes.data, b1 - b0)
        out = cuda.zeros(b1 - b0, dtype=cuda.uint8, device="cuda")
        prod.pack(td0.data_ptr() - lo, 1, tp, b0, out.data_ptr(), b1 - b0)
        cuda.cuda.synchronize()
        assert np.array_equal(td.cpu().numpy(), th), ("unpack", shape, b0, b1)
        assert np.array_equal(out.cpu().numpy(), ph), ("pack", shape, b0, b1)
    prod.type_free(tp)
    oracle.type_free(to)


def test_bad_shape_is_refused(shaped):
    assert shaped.lib.yaksa_gb300_debug_hidx_shape(7, 0, 0) == yk.ERR_INTERNAL
    assert shaped.lib.yaksa_gb300_debug_hidx_shape(0, 0, 99) == yk.ERR_INTERNAL


def test_tuned_repeats_are_exact(cuda, prod, oracle):
    """no shape forced: the autotuner times every candidate over the first launches of
    the class; every launch gives the oracle's bytes"""
    rng = np.random.default_rng(12)
    tp, to = _hindexed(prod, oracle, rng, 60000, 40, yk.TYPE_INT32_T, 4)
    n = prod.size(tp)
    lo, hi = _bounds(prod, tp)
    packed = rng.integers(0, 256, n, dtype=np.uint8)
    target = rng.integers(0, 256, hi - lo, dtype=np.uint8)
    th = target.copy()
    oracle.unpack(packed.ctypes.data, n, th.ctypes.data - lo, 1, to, 0)
    pd = dev_copy(cuda, packed)
    for i in range(40):
        td = dev_copy(cuda, target)
        prod.unpack(pd.data_ptr(), n, td.data_ptr() - lo, 1, tp, 0)
        cuda.cuda.synchronize()
        assert np.array_equal(td.cpu().numpy(), th), i
    prod.type_free(tp)
    oracle.type_free(to)
