"""GPU: the staging ring, for buffers the GPU cannot address in place.

On GB300 every host buffer is addressed in place, so the ring only runs when
YAKSA_GB300_HOST_DIRECT=0 turns in-place host access off.  That setting is read when the
library first brings the GPU up, so the cases run in a child process
(tests/staging_child.py) with a ring of 4 slabs of 64 KiB: 5 MiB requests take 80 chunks
and wrap the ring, 40 nonblocking requests are in flight at once (more than the ring
holds), the packed side, the typed side or both live in pageable or pinned host memory,
two cases unpack with SUM through overlaps into a staged typed buffer (double over
overlapping elements on the ordered kernel; int64 over overlapping indexed_block blocks,
folded in by L2 reductions on the staged device copy, checked by the library's launch
counter), and two
cases have an element larger than a slab.  Every result is compared byte for byte with
the oracle.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_staging_ring(cuda):
    env = dict(os.environ, YAKSA_GB300_HOST_DIRECT="0", YAKSA_GB300_STAGE_SLABS="4",
               YAKSA_GB300_STAGE_SLAB_KIB="64")
    r = subprocess.run([sys.executable, os.path.join(HERE, "staging_child.py")], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    bad = [k for k, v in res.items() if v is False]
    assert not bad, res
    # 18 single requests and 40 in flight, every one staged; none addressed in place
    assert res["staged_calls"] == 58 and res["direct_calls"] == 0, res


def test_wait_kernel_hint(cuda):
    """yaksa_init with yaksa_has_wait_kernel=true in a library told to stage every host
    buffer: pageable and pinned host buffers are used in place (no staging ring, whose
    pinned half would synchronize the device), and every result matches the oracle."""
    env = dict(os.environ, YAKSA_GB300_HOST_DIRECT="0")
    r = subprocess.run([sys.executable, os.path.join(HERE, "wait_kernel_child.py")], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    bad = [k for k, v in res.items() if v is False]
    assert not bad, res
    assert res["staged_calls"] == 0 and res["direct_calls"] == 4, res
