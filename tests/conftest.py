"""Shared test set-up: paths, the `gpu` marker, and on-demand builds.

CPU tests (`-m "not gpu"`) exercise the oracle, the golden fixtures and the
C-ABI host logic; GPU tests (`-m gpu`) run the CUDA library on cuda:0 and
compare it with the oracle.
"""
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "mpi-incompressible-fluid_gb300")
ORACLE = os.path.join(REPO, "oracle")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (PKG, ORACLE, REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built mifgpu library")


@pytest.fixture(scope="session")
def oracle_lib():
    """Build oracle/libmif_oracle.so (the C restatement) if needed."""
    subprocess.run(["make", "-s", "-C", ORACLE, "libmif_oracle.so"], check=True)
    import oracle

    return oracle


@pytest.fixture(scope="session")
def mifgpu_lib():
    """Build the CUDA library if needed and return the binding module."""
    import build as pkg_build

    pkg_build.build()
    import mifgpu

    mifgpu.load_library()
    return mifgpu


@pytest.fixture(scope="session")
def cuda_device():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
