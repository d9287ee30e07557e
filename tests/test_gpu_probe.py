"""The FP64 FMA-rate probe (instrumentation entry point, no reference
counterpart): it needs no context and returns a plausible positive rate."""
import math

import pytest

pytestmark = pytest.mark.gpu


def test_fp64_fma_probe_returns_a_rate(mifgpu_lib, cuda_device):
    rate = mifgpu_lib.probe_fp64_fma()
    assert math.isfinite(rate)
    # any CUDA GPU's FP64 FMA rate lies between 10 GFLOP/s and 1 PFLOP/s
    assert 0.01 < rate < 1000.0


def test_fp64_fma_probe_rejects_a_null_pointer(mifgpu_lib, cuda_device):
    lib = mifgpu_lib.load_library()
    assert lib.mifgpu_probe_fp64_fma(None) == -1
