"""ffs_measure_fp64_peak: the FP64 rates the FP64 roofline is stated against (positive;
one FMA does two flops, so the FMA rate in TFLOP/s exceeds the add rate)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_fp64_rates(gpu_pkg):
    L = gpu_pkg.load()
    fma, add = ctypes.c_double(), ctypes.c_double()
    assert L.ffs_measure_fp64_peak(0, ctypes.byref(fma), ctypes.byref(add)) == 0
    assert fma.value > 0 and add.value > 0
    assert add.value < fma.value
