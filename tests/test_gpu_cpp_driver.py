"""The reference's full-step convergence test (test/full_test.cpp) run as a
C++ program over the C++ host mirror (include/mifgpu.hpp), compared with the
oracle's norms and with the reference's expected velocity order 2
(analysis/plot_convergence.py:63-64)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu
DRIVER = os.path.join(REPO, "tests", "cpp", "full_test_gpu")


def run_driver(n, nt, mode="fp64"):
    out = subprocess.run([DRIVER, str(n), str(nt), mode], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    return np.array([float(x) for x in out.stdout.split()])


def oracle_norms(oracle_lib, n, nt):
    O = oracle_lib
    case = O.Case(n_global=(n, n, n), size=(1.0, 1.0, 2.0), origin=(0.0, 0.0, -1.0), Re=1e3, dt=1e-4 / nt,
                  exact_kind=O.KIND_ETHIER)
    s = O.OracleSolver(case)
    s.set_exact_velocity(0, 0.0, True)
    s.set_exact_pressure(0.0)
    for k in range(nt):
        s.timestep(k * case.dt)
    s.adjust_pressure(1e-4)
    return s.error_norms(1e-4)


def test_cpp_driver_matches_oracle_and_converges(oracle_lib, mifgpu_lib, cuda_device):
    if not os.path.exists(DRIVER):
        pytest.fail("tests/cpp/full_test_gpu not built (run __graft_entry__.build())")
    e17 = run_driver(17, 2)
    e33 = run_driver(33, 2)
    np.testing.assert_allclose(e17, oracle_norms(oracle_lib, 17, 2), rtol=1e-8)
    np.testing.assert_allclose(e33, oracle_norms(oracle_lib, 33, 2), rtol=1e-8)
    order = np.log2(e17[2] / e33[2])
    assert order > 1.7, order
    mixed = run_driver(33, 2, "mixed")
    assert abs(mixed[2] - e33[2]) <= 0.05 * e33[2]
