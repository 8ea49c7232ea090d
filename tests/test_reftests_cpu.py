"""CPU: the reference's own test programs.

The record in tests/golden/reftests_oracle.txt comes from oracle/run_reftests.py over the
reference's test matrix. The reference's pack, iov, flatten and simple programs ran
against the oracle; iov, lbub and test_contig also ran against the product library,
which they link unchanged. When those binaries were built on this machine
(`make -C oracle reftests`, which needs the reference tree), a few runs repeat live.
"""
import os
import platform
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RECORD = os.path.join(ROOT, "tests", "golden", "reftests_oracle.txt")
REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def test_record_has_every_program_and_no_failure():
    lines = [ln for ln in open(RECORD) if ln.startswith(("PASS", "FAIL"))]
    assert lines and all(ln.startswith("PASS") for ln in lines)
    progs = {}
    for ln in lines:
        prog = ln.split()[1]
        progs[prog] = progs.get(prog, 0) + 1
    assert progs["pack"] == 324
    assert progs["iov"] == 216 and progs["iov_product"] == 216
    assert progs["flatten"] == 36
    for p in ("simple_test", "threaded_test", "lbub", "test_contig", "lbub_product",
              "test_contig_product"):
        assert progs[p] == 1
    assert open(RECORD).read().rstrip().endswith(f"{len(lines)}/{len(lines)} passed")


ELF_MACHINE = {"x86_64": 0x3E, "aarch64": 0xB7}


def runnable(name):
    """The binary's path if it exists and was built for this machine (ELF e_machine)."""
    path = os.path.join(REF_BIN, name)
    if not os.path.exists(path):
        return None
    with open(path, "rb") as f:
        head = f.read(20)
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return None
    machine = int.from_bytes(head[18:20], "little")
    return path if ELF_MACHINE.get(platform.machine()) == machine else None


@pytest.mark.parametrize("args", [
    "-datatype short_int -count 1075 -seed 440 -iters 8 -segments 64 -ordering random -overlap none",
    "-datatype int:3+double:2 -count 17 -seed 441 -iters 64 -segments 64 -ordering normal -overlap irregular",
    "-datatype c_double_complex -count 65536 -seed 442 -iters 2 -segments 1 -ordering normal -overlap none",
])
def test_reference_iov_program_against_product(args):
    path = runnable("iov_product")
    if path is None:
        pytest.skip("reference test programs not built on this machine")
    r = subprocess.run([path] + args.split(), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
