"""Test configuration: the `gpu` marker and import paths.

CPU tests (-m "not gpu") cover the oracle against the reference's own pins and the golden
fixtures, the mesh generator, and the C ABI's exports and argument checks.  GPU tests
(-m gpu) are the parity tests proper: they call the CUDA library through its C ABI and
compare against the oracle and the golden fixtures.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "lpm-v2_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built_lib():
    """Builds liblpm_gpu.so (nvcc cross-compiles without a GPU) and returns the binding."""
    import build as pkg_build
    pkg_build.build()
    import lpm_gpu
    return lpm_gpu


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.lib()
    return oracle
