"""Test configuration: the `gpu` marker, import paths, shared fixtures.

`-m "not gpu"` runs the oracle checks against the committed golden fixtures, the ABI
symbol check and host-side logic; `-m gpu` runs the parity tests through the C ABI on a GPU.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bend-groth16_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests through the C ABI)")


@pytest.fixture(scope="session")
def built_lib():
    """libbg.so, brought up to date by make (nvcc cross-compiles without a GPU)."""
    import bendg
    import __graft_entry__
    __graft_entry__.build()
    return bendg.LIB_PATH


@pytest.fixture(scope="session")
def ctx(built_lib):
    import bendg
    c = bendg.Context(0)
    yield c
    c.close()
