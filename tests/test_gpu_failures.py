"""GPU: failures surface as the reference's return codes and leave the library usable,
with every failure made on the host (no GPU fault, trap or hang is involved):

- an allocation that fails (injected with yaksa_gb300_debug_fail_alloc) returns
  YAKSA_ERR__OUT_OF_MEM, and the same call succeeds, bit-exact, once memory is back (a
  failed descriptor build is not cached);
- a request server that cannot get its rings is not created, and the next one is;
- an unknown type handle is YAKSA_ERR__INTERNAL, and long double arithmetic, which has no
  GPU form, is YAKSA_ERR__NOT_SUPPORTED.
"""
import numpy as np
import pytest

import yaksa_gb300 as yk
from helpers import dev_copy, fill, host_of

pytestmark = pytest.mark.gpu


def test_descriptor_allocation_failure_is_reported_and_retried(cuda, prod, oracle):
    rng = np.random.default_rng(8)
    blens = rng.integers(1, 20, 500).tolist()
    displs = (np.cumsum(np.array(blens) + 3) * 4).tolist()
    tp = prod.type_create_hindexed(blens, displs, yk.TYPE_INT32_T)
    to = oracle.type_create_hindexed(blens, displs, yk.TYPE_INT32_T)
    n = prod.size(tp)
    typed = fill(rng, displs[-1] + 4 * blens[-1] + 64, "int32")
    tg = dev_copy(cuda, typed)
    pg = cuda.zeros(n, dtype=cuda.uint8, device="cuda")
    prod.lib.yaksa_gb300_debug_fail_alloc(1)
    with pytest.raises(yk.YaksaError) as e:
        prod.pack(tg.data_ptr(), 1, tp, 0, pg.data_ptr(), n)
    assert e.value.rc == yk.ERR_OUT_OF_MEM
    assert prod.pack(tg.data_ptr(), 1, tp, 0, pg.data_ptr(), n) == n
    cuda.cuda.synchronize()
    expect = np.zeros(n, dtype=np.uint8)
    oracle.pack(typed.ctypes.data, 1, to, 0, expect.ctypes.data, n)
    assert np.array_equal(host_of(cuda, pg), expect)
    prod.type_free(tp)
    oracle.type_free(to)


def test_server_creation_failure(prod):
    prod.lib.yaksa_gb300_debug_fail_alloc(1)
    with pytest.raises(yk.YaksaError) as e:
        yk.Server(prod, ring_requests=8)
    assert e.value.rc == yk.ERR_OUT_OF_MEM
    srv = yk.Server(prod, ring_requests=8)
    srv.destroy()


def test_bad_handle_and_unsupported_operator(cuda, prod):
    buf = cuda.zeros(64, dtype=cuda.uint8, device="cuda")
    with pytest.raises(yk.YaksaError) as e:
        prod.pack(buf.data_ptr(), 1, 123456789, 0, buf.data_ptr(), 64)
    assert e.value.rc == yk.ERR_INTERNAL
    t = prod.type_create_contig(2, yk.TYPE_LONG_DOUBLE)
    if np.finfo(np.longdouble).nmant == 112:
        # binary128 long double: the GPU computes it (test_gpu_long_double.py)
        assert prod.unpack(buf.data_ptr(), 32, buf.data_ptr() + 32, 1, t, 0, op=yk.OP_SUM) == 32
    else:
        # another long double format (x87): no GPU form of its arithmetic
        with pytest.raises(yk.YaksaError) as e:
            prod.unpack(buf.data_ptr(), 32, buf.data_ptr(), 1, t, 0, op=yk.OP_SUM)
        assert e.value.rc == yk.ERR_NOT_SUPPORTED
    # REPLACE of the same data is a byte copy and works
    assert prod.unpack(buf.data_ptr(), 32, buf.data_ptr() + 32, 1, t, 0) == 32
    prod.type_free(t)
