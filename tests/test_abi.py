"""CPU: the C-ABI libraries load and export every function the public headers declare,
and the builtin handle values are the reference's (src/frontend/include/yaksa.h.in)."""
import ctypes
import os
import re

import pytest

import yaksa_gb300 as yk
from conftest import ROOT, _ensure_oracle, _ensure_product


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*int\s+(yaksa\w+)\s*\(", text, flags=re.M)))


def test_header_declares_reference_api():
    fns = declared_functions("yaksa.h")
    # the 34 public functions of yaksa.h.in:221-634 (pack_stream/unpack_stream included)
    assert len(fns) == 34, fns


@pytest.mark.parametrize("header", ["yaksa.h", "yaksa_gb300.h"])
def test_product_exports_declared_symbols(header):
    lib = ctypes.CDLL(_ensure_product(), mode=os.RTLD_LOCAL)
    for fn in declared_functions(header):
        assert hasattr(lib, fn), fn


def test_oracle_exports_reference_api():
    lib = ctypes.CDLL(_ensure_oracle(), mode=os.RTLD_LOCAL)
    for fn in declared_functions("yaksa.h"):
        assert hasattr(lib, fn), fn


def test_handle_constants_match_reference():
    text = open(os.path.join(ROOT, "include", "yaksa.h")).read()
    vals = dict((m.group(1), int(m.group(2))) for m in
                re.finditer(r"#define YAKSA_TYPE__(\w+)\s+\(\(yaksa_type_t\) (\d+)\)", text))
    assert vals["NULL"] == 0 and vals["_BOOL"] == 1 and vals["INT32_T"] == 8
    assert vals["FLOAT"] == 45 and vals["C_COMPLEX"] == 48 and vals["LONG_DOUBLE_INT"] == 56
    assert sorted(vals.values()) == list(range(57))
    ops = dict((m.group(1), int(m.group(2))) for m in
               re.finditer(r"#define YAKSA_OP__(\w+)\s+\(\(yaksa_op_t\) (\d+)\)", text))
    assert ops == {"MAX": 0, "MIN": 1, "SUM": 2, "PROD": 3, "LAND": 4, "BAND": 5, "LOR": 6,
                   "BOR": 7, "LXOR": 8, "BXOR": 9, "REPLACE": 10, "LAST": 11}


def test_product_has_no_cpu_path(prod):
    """Without a GPU the engine refuses pack/unpack loudly instead of computing on the CPU."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    buf = (ctypes.c_double * 16)()
    out = (ctypes.c_double * 16)()
    t = prod.type_create_vector(4, 1, 2, yk.TYPE_DOUBLE)
    with pytest.raises(yk.YaksaError) as e:
        prod.pack(ctypes.addressof(buf), 1, t, 0, ctypes.addressof(out), 128)
    assert e.value.rc == yk.ERR_INTERNAL
    prod.type_free(t)
