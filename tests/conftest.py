"""pytest configuration: the `gpu` marker, and session fixtures for the GPU engine
(libyaksa.so) and the CPU oracle (oracle/_ref/liboracle_yaksa.so)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

ORACLE_LIB = os.path.join(ROOT, "oracle", "_ref", "liboracle_yaksa.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity against the CPU oracle)")


def _ensure_oracle():
    if not os.path.exists(ORACLE_LIB):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return ORACLE_LIB


def _ensure_product():
    import yaksa_gb300
    if not os.path.exists(yaksa_gb300.LIB_PATH):
        from yaksa_gb300 import build
        build.build()
    return yaksa_gb300.LIB_PATH


@pytest.fixture(scope="session")
def oracle():
    import yaksa_gb300 as yk
    y = yk.Yaksa(_ensure_oracle())
    y.init()
    yield y
    y.finalize()


@pytest.fixture(scope="session")
def prod():
    import yaksa_gb300 as yk
    y = yk.Yaksa(_ensure_product())
    y.init()
    yield y
    y.finalize()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
