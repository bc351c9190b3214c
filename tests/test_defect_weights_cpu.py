"""The defect-repair weight w1 = (m+1)/(len+1): the reference rounds the double
quotient to float; the device kernels use one IEEE float division. Check that
both give the same bits for every run that fits a detector ring of up to 8192
columns (runs of length up to 8193 in the reference's wrap-around case)."""
import numpy as np


def test_float_division_equals_rounded_double_quotient():
    for length in range(1, 8194):
        m1 = np.arange(1, length + 1, dtype=np.float64)
        via_double = (m1 / float(length + 1)).astype(np.float32)
        via_float = m1.astype(np.float32) / np.float32(length + 1)
        assert np.array_equal(via_double.view(np.uint32), via_float.view(np.uint32)), length
