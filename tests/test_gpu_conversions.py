"""The integer-operation conversions of the light refresh (in place of FP64
instructions, which GB300 runs at a small fraction of its FP32 rate) give
the hardware's results bit for bit."""
import ctypes

import pytest
import torch

from pysph_gb300 import native

pytestmark = pytest.mark.gpu


def test_integer_conversions_match_the_hardware():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    out = ctypes.c_int64(-1)
    native.check(native.lib().sph_selftest_conversions(1 << 24, ctypes.byref(out)),
                 "sph_selftest_conversions")
    assert out.value == 0
