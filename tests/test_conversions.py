"""The integer-pipe FP64 <-> FP32 conversions of the FP32-stencil Cahn-Hilliard variant give exactly the
hardware conversions' results (round to nearest even one way, exact the other), on 2^30 seeded values of
each kind: random encodings, values at both ends of the float range, halfway cases and zeros."""
import ctypes

import pytest

import custen_gb300 as cs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2])
def test_integer_conversions_equal_hardware(gpu, seed):
    bad = ctypes.c_ulonglong(99)
    rc = cs.lib().custen_selftest_conversions(ctypes.c_ulonglong(1 << 30), ctypes.c_ulonglong(seed),
                                              ctypes.byref(bad))
    assert rc == 0
    assert bad.value == 0
