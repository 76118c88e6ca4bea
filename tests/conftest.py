"""Shared test set-up: the `gpu` marker, import paths and checker fixtures.

CPU tests (`-m "not gpu"`) check the oracle against the reference's golden
vectors and known answers, the host logic and the C ABI's exports. GPU tests
(`-m gpu`) run the CUDA path through the C ABI and compare it with the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "hpc-reading-course_gb300")
for p in (os.path.join(ROOT, "oracle"), os.path.join(PKG, "python"), PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def port():
    import oracle

    oracle.build()
    return oracle.Port()


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "ref_rhs.npz"))


@pytest.fixture(scope="session")
def sbp():
    """The CUDA library's binding, built in tree; fails loudly if it cannot be built."""
    import build as gpu_build

    gpu_build.build()
    import sbpgpu

    sbpgpu.load()
    return sbpgpu
