"""Child process of test_gpu_staging.py::test_wait_kernel_hint: the library started with
YAKSA_GB300_HOST_DIRECT=0 (stage every host buffer) and initialised with the
yaksa_has_wait_kernel hint.  The hint means the caller may keep a kernel resident that
waits on the host, so the library must not pin staging memory (cudaHostAlloc
synchronizes the device); host buffers the GPU can address are then used in place, as
the reference treats unregistered host buffers as registered under the same hint
(src/backend/src/yaksuri_progress.c:17-27).  Prints one JSON line: a verdict per case
(bytes against the oracle) and the library's staged and in-place call counts.
"""
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

import yaksa_gb300 as yk  # noqa: E402
from conftest import _ensure_oracle, _ensure_product  # noqa: E402


def main():
    prod = yk.Yaksa(_ensure_product())
    orc = yk.Yaksa(_ensure_oracle())
    info = prod.info_create(yaksa_has_wait_kernel="true")
    prod.init(info)
    prod.info_free(info)
    orc.init()
    rng = np.random.default_rng(43)
    out = {}
    s0 = prod.stats()
    tp = prod.type_create_hvector(20000, 4, 48, yk.TYPE_DOUBLE)
    to = orc.type_create_hvector(20000, 4, 48, yk.TYPE_DOUBLE)
    n = prod.size(tp)
    typed0 = rng.standard_normal(20000 * 6).view(np.uint8)
    packed0 = rng.standard_normal(n // 8).view(np.uint8)
    for where in ("pageable", "pinned"):
        # pack: typed on the device, packed into host memory; unpack: the reverse
        td = torch.from_numpy(typed0.copy()).cuda()
        torch.cuda.synchronize()
        if where == "pinned":
            ph_t = torch.zeros(n, dtype=torch.uint8).pin_memory()
            ph, get = ph_t.data_ptr(), lambda: ph_t.numpy().copy()
        else:
            ph_a = np.zeros(n, dtype=np.uint8)
            ph, get = ph_a.ctypes.data, lambda: ph_a.copy()
        got, req = prod.ipack(td.data_ptr(), 1, tp, 0, ph, n)
        prod.wait(req)
        ref = np.zeros(n, dtype=np.uint8)
        orc.pack(typed0.ctypes.data, 1, to, 0, ref.ctypes.data, n)
        out[f"pack_into_{where}"] = bool(got == n and np.array_equal(get(), ref))
        th = typed0.copy() if where == "pageable" else None
        tt = torch.from_numpy(typed0.copy()).pin_memory() if where == "pinned" else None
        tptr = th.ctypes.data if th is not None else tt.data_ptr()
        pd = torch.from_numpy(packed0.copy()).cuda()
        torch.cuda.synchronize()
        got, req = prod.iunpack(pd.data_ptr(), n, tptr, 1, tp, 0, op=yk.OP_SUM)
        prod.wait(req)
        exp = typed0.copy()
        orc.unpack(packed0.ctypes.data, n, exp.ctypes.data, 1, to, 0, op=yk.OP_SUM)
        res = th if th is not None else tt.numpy()
        out[f"unpack_sum_into_{where}"] = bool(got == n and np.array_equal(res, exp))
    s1 = prod.stats()
    out["staged_calls"] = s1["staged_calls"] - s0["staged_calls"]
    out["direct_calls"] = s1["direct_calls"] - s0["direct_calls"]
    prod.type_free(tp)
    orc.type_free(to)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
