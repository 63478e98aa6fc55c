"""The sm_103a WENO5 advection operator (cuStenCreate2DXYWENOADVp / Compute / Swap / Destroy): bit for
bit against the reference's own kernel on the same GPU (both call CUDA's powf), and against the CPU
oracle within the float precision of the powf terms (GPU)."""
import ctypes

import numpy as np
import pytest

import custen_gb300 as cs
import oracle
from custen_gb300.buffers import DeviceBuffer, HostBuffer
from custen_gb300.inputs import weno_inputs
from tests.test_weno_oracle import weno_close

pytestmark = pytest.mark.gpu


def run_weno(nx, ny, tiles, seed, rough=False, mem="device", offload=cs.DEVICE, bx=32, by=8):
    f, u, v, dx, dy = weno_inputs(nx, ny, seed, rough=rough)
    pre = np.full((ny, nx), 7.0)
    if mem == "device" or mem == "managed":
        bufs = [DeviceBuffer.from_array(a, mem == "managed") for a in (f, u, v, pre)]
    else:
        bufs = [HostBuffer.from_array(a) for a in (f, u, v, pre)]
    h = cs.WenoAdvection(nx, ny, bufs[3].ptr, bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, dx=dx, dy=dy, num_tiles=tiles,
                         block_x=bx, block_y=by)
    h.compute(offload)
    cs._check(cs.lib().custen_device_synchronize())
    if mem == "device":
        got = bufs[3].download((ny, nx), np.float64)
    else:
        got = bufs[3].view((ny, nx), np.float64).copy()
    h.destroy()
    return got, oracle.weno(f, u, v, 1.0 / dx, 1.0 / dy)


def assert_same(got, ref):
    bad = got != ref
    assert not bad.any(), f"{bad.sum()} of {bad.size} points differ; first {np.argwhere(bad)[:3].tolist()}"


def assert_close(got, ref):
    ok, err = weno_close(got, ref)
    assert ok, f"rel L2 {err[0]:.2e}, rel max {err[1]:.2e}"


def reference_out(nx, ny, tiles, bx, by, seed, rough):
    """The reference kernel's output for the same inputs, or None without the reference cubin."""
    if oracle.reference_kernels() is None:
        return None
    f, u, v, dx, dy = weno_inputs(nx, ny, seed, rough=rough)
    bufs = [DeviceBuffer.from_array(a) for a in (f, u, v)]
    out = DeviceBuffer.from_array(np.zeros_like(f))
    oracle.reference_weno(nx, ny, tiles, bx, by, out.ptr, bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, 1 / dx, 1 / dy)
    return out.download((ny, nx), np.float64)


# (nx, ny, numTiles, BLOCK_X, BLOCK_Y): the reference kernel's preconditions hold (nx % BLOCK_X == 0,
# nyTile % BLOCK_Y == 0, two or more blocks per direction and tile)
REF_SHAPES = [(64, 64, 1, 16, 8), (128, 96, 3, 32, 16), (256, 128, 4, 32, 8), (96, 64, 2, 16, 16)]


@pytest.mark.parametrize("shape", REF_SHAPES)
@pytest.mark.parametrize("rough", [False, True])
def test_weno_bit_identical_to_reference_kernel(gpu, shape, rough):
    nx, ny, tiles, bx, by = shape
    seed = nx + ny + tiles
    ref = reference_out(nx, ny, tiles, bx, by, seed, rough)
    if ref is None:
        pytest.skip("reference cubin not present")
    got, ora = run_weno(nx, ny, tiles, seed=seed, rough=rough, bx=bx, by=by)
    assert_same(got, ref)
    assert_close(got, ora)


@pytest.mark.parametrize("nx,ny,tiles", [(64, 64, 1), (128, 96, 3), (100, 70, 2), (40, 36, 1), (200, 66, 2)])
@pytest.mark.parametrize("rough", [False, True])
def test_weno_matches_oracle(gpu, nx, ny, tiles, rough):
    """Any size, including partial 64 x 32 tiles and shapes the reference kernel cannot run."""
    got, ref = run_weno(nx, ny, tiles, seed=nx + ny + tiles, rough=rough)
    assert_close(got, ref)


@pytest.mark.parametrize("tiles", [1, 4])
@pytest.mark.parametrize("mem", ["pinned", "managed"])
def test_weno_host_resident_fields(gpu, tiles, mem):
    """Pinned fields stream through the staging slots (velocity rows included, chunks of a few rows);
    managed fields take the prefetch path; HOST offload."""
    cs.set_stage_chunk_bytes(4096)
    try:
        got, ref = run_weno(64, 128, tiles, seed=3, rough=True, mem=mem, offload=cs.HOST, bx=16, by=8)
    finally:
        cs.set_stage_chunk_bytes(0)
    assert_close(got, ref)


def test_weno_swap_and_coefficients_read_per_compute(gpu):
    """Compute, Swap (halo pointers re-derived from the new input), Compute again; then coeDx changed
    in the handle between Computes is honoured (the reference passes it at every launch)."""
    nx, ny, tiles = 64, 96, 3
    f, u, v, dx, dy = weno_inputs(nx, ny, 11)
    A = DeviceBuffer.from_array(np.zeros_like(f))
    Bf = DeviceBuffer.from_array(f)
    U, V = DeviceBuffer.from_array(u), DeviceBuffer.from_array(v)
    h = cs.WenoAdvection(nx, ny, A.ptr, Bf.ptr, U.ptr, V.ptr, dx=dx, dy=dy, num_tiles=tiles, block_x=16, block_y=8)
    h.compute(cs.DEVICE)
    h.swap(A.ptr)
    h.compute(cs.DEVICE)
    cs._check(cs.lib().custen_device_synchronize())
    got1 = A.download((ny, nx), np.float64)
    assert_close(got1, oracle.weno(f, u, v, 1 / dx, 1 / dy))
    got2 = Bf.download((ny, nx), np.float64)
    assert_close(got2, oracle.weno(got1, u, v, 1 / dx, 1 / dy))
    t = cs.CuStenT.from_buffer(h.handle)
    assert t.coeDx == 1.0 / dx and t.coeDy == 1.0 / dy
    t.coeDx = 2.0 / dx
    h.swap(Bf.ptr)
    h.compute(cs.DEVICE)
    cs._check(cs.lib().custen_device_synchronize())
    assert_close(A.download((ny, nx), np.float64), oracle.weno(got2, u, v, 2 / dx, 1 / dy))
    h.destroy()


def test_weno_create_rejects_bad_arguments(gpu):
    buf = DeviceBuffer(64 * 64 * 8)
    hb = ctypes.create_string_buffer(cs.HANDLE_BYTES)
    L = cs.lib()
    assert L.custen_create_2d_xyweno_adv_p(hb, 0, 1, 64, 64, 16, 8, 0.1, 0.1, None, buf.ptr, buf.ptr, buf.ptr) == 2
    assert L.custen_create_2d_xyweno_adv_p(hb, 0, 32, 64, 64, 16, 2, 0.1, 0.1, buf.ptr, buf.ptr, buf.ptr,
                                           buf.ptr) == 2   # 2 rows per tile < 3
    assert L.custen_create(hb, cs.XYWENOADVP, cs.F64, 0, 1, 64, 64, 16, 8, buf.ptr, buf.ptr, buf.ptr, 7, 3, 3, 7, 3,
                           3, 0, None) == 2
