"""The allocation-free Cahn-Hilliard step, checked against the regular batch entry point (GPU).

custen_ch_step_noalloc exists for callers that cannot allocate device memory: a plug-in inside a
host application that owns all device memory through its own budgeted pool, or a loop that must not
enter cudaMalloc / cudaFree because they synchronise the device. It keeps its work buffers in a
static device array of the library (grids up to 256 x 256). This file is collected last so that a
run stopping at the first failure has already run every other test; it also passes on its own.
"""
import ctypes
import math

import numpy as np
import pytest

import custen_gb300 as cs
from custen_gb300.buffers import DeviceBuffer

pytestmark = pytest.mark.gpu

REL_L2 = 1e-10   # the tolerance of the Cahn-Hilliard parity tests


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _batch_two_steps(n, c0):
    b = cs.CahnHilliardBatch([n])
    b.set_state(0, c0)
    b.step(1, graph=False)
    r1 = b.state(0)[0]
    b.step(1, graph=False)
    r2 = b.state(0)[0]
    b.close()
    return r1, r2


@pytest.mark.parametrize("n", [64, 128, 256])
def test_noalloc_two_calls_match_batch_entry_point(gpu, n):
    """Two calls in a row, three distinct buffers, up to the largest allowed grid (whose field fills the
    whole work region of the static array). Every kernel configuration of the solver computes the same
    values, so the fields must equal the batch entry point's bit for bit (which is within REL_L2)."""
    c0 = np.random.default_rng(9 + n).uniform(-0.1, 0.1, (n, n))
    L = cs.lib()
    d_old, d_cur = DeviceBuffer.from_array(c0), DeviceBuffer.from_array(c0)
    d_new = DeviceBuffer(n * n * 8)
    # call 1: (cOld, cCurr) = (c0, c0) -> c1 in d_new
    rc = L.custen_ch_step_noalloc(d_old.ptr, d_cur.ptr, d_new.ptr, n, 2 * math.pi, 0.01, 0.1, None)
    assert rc == 0, L.custen_ch_last_error()
    assert L.custen_device_synchronize() == 0
    c1 = d_new.download((n, n), np.float64)
    # call 2: (cOld, cCurr) = (c0, c1) -> c2, written over the c0 buffer that served as cOld
    rc = L.custen_ch_step_noalloc(d_cur.ptr, d_new.ptr, d_old.ptr, n, 2 * math.pi, 0.01, 0.1, None)
    assert rc == 0, L.custen_ch_last_error()
    assert L.custen_device_synchronize() == 0
    c2 = d_old.download((n, n), np.float64)

    r1, r2 = _batch_two_steps(n, c0)
    assert _rel(c1, r1) <= REL_L2 and _rel(c2, r2) <= REL_L2
    assert np.array_equal(c1, r1)
    assert np.array_equal(c2, r2)


@pytest.mark.parametrize("n", [64, 256])
def test_noalloc_in_place_over_c_old(gpu, n):
    """c_new given as the c_old buffer (the documented in-place form), two calls in a row rotating two
    buffers: equal to the batch entry point bit for bit."""
    c0 = np.random.default_rng(19 + n).uniform(-0.1, 0.1, (n, n))
    L = cs.lib()
    a, b = DeviceBuffer.from_array(c0), DeviceBuffer.from_array(c0)
    # call 1: (cOld, cCurr) = (a, b) = (c0, c0) -> c1 written over a
    rc = L.custen_ch_step_noalloc(a.ptr, b.ptr, a.ptr, n, 2 * math.pi, 0.01, 0.1, None)
    assert rc == 0, L.custen_ch_last_error()
    # call 2: (cOld, cCurr) = (b, a) = (c0, c1) -> c2 written over b
    rc = L.custen_ch_step_noalloc(b.ptr, a.ptr, b.ptr, n, 2 * math.pi, 0.01, 0.1, None)
    assert rc == 0, L.custen_ch_last_error()
    assert L.custen_device_synchronize() == 0
    c1 = a.download((n, n), np.float64)
    c2 = b.download((n, n), np.float64)
    r1, r2 = _batch_two_steps(n, c0)
    assert np.array_equal(c1, r1)
    assert np.array_equal(c2, r2)


def test_noalloc_rejects_c_new_aliasing_c_cur(gpu):
    n = 64
    L = cs.lib()
    a, b = DeviceBuffer(n * n * 8), DeviceBuffer(n * n * 8)
    rc = L.custen_ch_step_noalloc(a.ptr, b.ptr, b.ptr, n, 2 * math.pi, 0.01, 0.1, None)
    assert rc == 2
    assert b"c_cur" in L.custen_ch_last_error()


def test_noalloc_rejects_grids_above_its_maximum(gpu):
    n = 288
    L = cs.lib()
    buf = DeviceBuffer(8 * 64)
    rc = L.custen_ch_step_noalloc(buf.ptr, buf.ptr + 8, buf.ptr + 16, n, 2 * math.pi, 0.01, 0.1, None)
    assert rc == 2
    assert b"maximum of 256" in L.custen_ch_last_error()
