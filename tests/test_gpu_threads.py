"""GPU: the library is thread safe, as the reference's is (test/simple/threaded_test.c runs
16 threads).  Eight host threads create and free their own types and run blocking,
nonblocking and stream-ordered packs and unpacks at the same time; every result matches
the oracle's, computed beforehand on the same inputs.

Tolerance: byte-identical (REPLACE).
"""
import ctypes
import threading

import numpy as np
import pytest

from helpers import fill
from typegen import Gen, build, footprint

pytestmark = pytest.mark.gpu

NTHREADS, ITERS = 8, 12


def test_concurrent_threads_match_oracle(cuda, prod, oracle):
    # inputs and expected results, prepared serially
    work = []
    g = Gen(oracle, 77, max_depth=3)
    rng = np.random.default_rng(77)
    for t in range(NTHREADS):
        items = []
        for i in range(ITERS):
            base = ["int32", "double", "int8", "float"][(t + i) % 4]
            r = g.gen(base)
            ko = []
            ho = build(oracle, r, ko)
            count = int(rng.integers(1, 4))
            lo, hi, size = footprint(oracle, ho, count)
            typed = fill(rng, hi - lo + 64, base)
            packed = np.zeros(size * count, dtype=np.uint8)
            oracle.pack(typed.ctypes.data + 32 - lo, count, ho, 0, packed.ctypes.data, size * count)
            back = np.zeros_like(typed)
            oracle.unpack(packed.ctypes.data, size * count, back.ctypes.data + 32 - lo, count, ho, 0)
            for h in reversed(ko):
                oracle.type_free(h)
            items.append(dict(r=r, count=count, lo=lo, size=size, typed=typed, packed=packed,
                              back=back, mode=i % 3))
        work.append(items)
    g.free()
    errors = []

    def worker(items):
        try:
            stream = cuda.cuda.Stream()
            sh = ctypes.c_void_p(stream.cuda_stream)
            for it in items:
                keep = []
                h = build(prod, it["r"], keep)
                n = it["size"] * it["count"]
                tg = cuda.from_numpy(it["typed"]).cuda()
                pg = cuda.zeros(n, dtype=cuda.uint8, device="cuda")
                bg = cuda.zeros(len(it["typed"]), dtype=cuda.uint8, device="cuda")
                cuda.cuda.synchronize()
                tp, bp = tg.data_ptr() + 32 - it["lo"], bg.data_ptr() + 32 - it["lo"]
                if it["mode"] == 0:
                    prod.pack(tp, it["count"], h, 0, pg.data_ptr(), n)
                    prod.unpack(pg.data_ptr(), n, bp, it["count"], h, 0)
                elif it["mode"] == 1:
                    prod.wait(prod.ipack(tp, it["count"], h, 0, pg.data_ptr(), n)[1])
                    prod.wait(prod.iunpack(pg.data_ptr(), n, bp, it["count"], h, 0)[1])
                else:
                    prod.pack_stream(tp, it["count"], h, 0, pg.data_ptr(), n, ctypes.addressof(sh))
                    prod.unpack_stream(pg.data_ptr(), n, bp, it["count"], h, 0, ctypes.addressof(sh))
                    stream.synchronize()
                for k in reversed(keep):
                    prod.type_free(k)
                if not np.array_equal(pg.cpu().numpy(), it["packed"]):
                    errors.append(("packed", it["r"]))
                if not np.array_equal(bg.cpu().numpy(), it["back"]):
                    errors.append(("unpacked", it["r"]))
        except Exception as e:     # reported by the main thread
            errors.append(("exception", repr(e)))

    threads = [threading.Thread(target=worker, args=(w,)) for w in work]
    for th in threads:
        th.start()
    for th in threads:
        th.join(timeout=300)
    assert not any(th.is_alive() for th in threads)
    assert not errors, errors[:4]


@pytest.mark.parametrize("nstreams", ["1", "16"])
def test_library_stream_counts(cuda, nstreams):
    """The threaded test and the nonblocking parity tests again, in a child process, with
    one library stream (every request in one order) and with sixteen."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-p", "no:cacheprovider",
                        os.path.join(here, "test_gpu_threads.py"), os.path.join(here, "test_gpu_parity.py"),
                        "-k", "concurrent_threads or nonblocking or host_buffers"],
                       env=dict(os.environ, YAKSA_GB300_LIB_STREAMS=nstreams),
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
