"""ffs_measure_fp64_peak and ffs_measure_fp64_register_rate: the FP64 rates the FP64
roofline is stated against (positive, and the register-operand FMA rate no faster than
the constant-operand one)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_fp64_rates(gpu_pkg):
    L = gpu_pkg.load()
    fma, add, reg = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    assert L.ffs_measure_fp64_peak(0, ctypes.byref(fma), ctypes.byref(add)) == 0
    assert L.ffs_measure_fp64_register_rate(0, ctypes.byref(reg)) == 0
    assert fma.value > 0 and add.value > 0 and reg.value > 0
    assert reg.value <= 1.05 * fma.value
