"""The winding-number kernels divide several numerators by one denominator
with Markstein's method (one correctly rounded reciprocal, then a product and
a fused correction per quotient).  Inside the range those kernels guard
(dividends and divisors within [2^-60, 2^60]) every step scales exactly with
the operands' exponents, so the method equals IEEE division there exactly
when it does on every pair of significands: this test checks all 2^46 pairs
on the GPU against CUDA's __fdiv_rn."""
import ctypes

import pytest

from baby_shark_gb300 import _native as N
from tests.gpu_common import context

pytestmark = pytest.mark.gpu


def test_shared_reciprocal_division_is_ieee_on_every_significand_pair():
    ctx = context()
    bad, tested = ctypes.c_uint64(), ctypes.c_uint64()
    N.check(N.load().bs_diag_check_division(ctx.h, 1, ctypes.byref(bad), ctypes.byref(tested)), ctx.h)
    assert tested.value == 1 << 46
    assert bad.value == 0
