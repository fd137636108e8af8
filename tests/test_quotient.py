"""The interface Riemann solver's shared-reciprocal quotients (Markstein's
method, m2cg_device.cuh: quot_of / qdiv) must equal IEEE division bit for bit,
so that the device solver follows the oracle's operations exactly.  The check
runs on the device over 2^32 operand pairs of every class the self-test draws
(random bit patterns, wide and physical exponent ranges, all-ones significands,
zeros, subnormals, infinities, NaNs, exponent-limit and exact quotients)."""
import ctypes as C

import pytest

from m2c_gb300 import abi

INVALID_ARG = 1   # M2CG_ERR_INVALID_ARG


def test_selftest_entry_rejects_bad_arguments():
    lib = abi.load()
    bad = C.c_int64(-1)
    assert lib.m2cg_selftest_quotient(0, 1, C.byref(bad), None) == INVALID_ARG
    assert lib.m2cg_selftest_quotient(1 << 37, 1, C.byref(bad), None) == INVALID_ARG
    assert lib.m2cg_selftest_quotient(16, 1, None, None) == INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 20261204])
def test_shared_reciprocal_quotients_equal_ieee_division(seed):
    lib = abi.load()
    bad, fast = C.c_int64(-1), C.c_int64(-1)
    n = 1 << 32
    abi.check(lib, lib.m2cg_selftest_quotient(n, seed, C.byref(bad), C.byref(fast)), "m2cg_selftest_quotient")
    assert bad.value == 0
    # most operand classes are inside the shared-reciprocal path's range
    assert 0.4 * n < fast.value < n
