"""Shared test helpers: seeded fields, device buffers through the library's C-ABI, configs."""
from __future__ import annotations

import ctypes

import numpy as np

import custen_gb300 as cs


class DeviceBuffer:
    """Device (or managed) allocation made through the C-ABI (no torch needed)."""

    def __init__(self, nbytes: int, managed: bool = False):
        self.nbytes = nbytes
        self.managed = managed
        p = ctypes.c_void_p()
        fn = cs.lib().custen_malloc_managed if managed else cs.lib().custen_malloc_device
        cs._check(fn(ctypes.byref(p), max(nbytes, 16)))
        self.ptr = int(p.value)

    @classmethod
    def from_array(cls, a: np.ndarray, managed: bool = False) -> "DeviceBuffer":
        b = cls(a.nbytes, managed)
        b.upload(a)
        return b

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        cs._check(cs.lib().custen_memcpy(self.ptr, a.ctypes.data, a.nbytes))

    def download(self, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        cs._check(cs.lib().custen_memcpy(out.ctypes.data, self.ptr, out.nbytes))
        return out

    def view(self, shape, dtype) -> np.ndarray:
        """Host view of managed memory (valid after a device synchronize)."""
        assert self.managed
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        buf = (ctypes.c_char * n).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            cs.lib().custen_free(self.ptr)
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class HostBuffer:
    """Pinned host allocation made through the C-ABI, with a numpy view."""

    def __init__(self, nbytes: int):
        self.nbytes = nbytes
        p = ctypes.c_void_p()
        cs._check(cs.lib().custen_malloc_host(ctypes.byref(p), max(nbytes, 16)))
        self.ptr = int(p.value)

    @classmethod
    def from_array(cls, a: np.ndarray) -> "HostBuffer":
        b = cls(a.nbytes)
        b.view(a.shape, a.dtype)[...] = a
        return b

    def view(self, shape, dtype) -> np.ndarray:
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        assert n <= self.nbytes
        buf = (ctypes.c_char * n).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            cs.lib().custen_free_host(self.ptr)
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def field(nx: int, ny: int, seed: int, dtype=np.float64) -> np.ndarray:
    """sin(3x)cos(5y) + U(-1e-3, 1e-3) on [0,2pi)^2 (the benchmark field)."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * (2 * np.pi / nx)
    y = np.arange(ny) * (2 * np.pi / ny)
    f = np.sin(3 * x)[None, :] * np.cos(5 * y)[:, None] + rng.uniform(-1e-3, 1e-3, size=(ny, nx))
    return np.ascontiguousarray(f.astype(dtype))


def weights_for(variant: int, H: int, V: int, seed: int, dtype=np.float64, zeros: bool = True) -> np.ndarray:
    rng = np.random.default_rng(1000 + seed)
    w = rng.uniform(-2.0, 2.0, size=H * V)
    if zeros and H * V >= 4:
        w[rng.choice(H * V, size=max(1, H * V // 4), replace=False)] = 0.0
    return w.astype(dtype)


def sentinel(nx: int, ny: int, dtype=np.float64) -> np.ndarray:
    """Pre-fill of the output: distinct, finite, recognisable values."""
    return (np.arange(nx * ny, dtype=np.float64).reshape(ny, nx) * 1e-3 + 12345.0).astype(dtype)


def weno_inputs(nx: int, ny: int, seed: int, rough: bool = False):
    """Advected field, velocities and spacings for the WENO operator: the benchmark field (or, rough,
    a random one that drives the nonlinear weights), u and v of both signs with some exact zeros (the
    reference's `> 0.0` test sends them to the other upwind side), dx = 2 pi / nx, dy = 2 pi / ny."""
    rng = np.random.default_rng(500 + seed)
    f = rng.standard_normal((ny, nx)) if rough else field(nx, ny, seed)
    u = rng.uniform(-1.0, 1.0, (ny, nx))
    v = rng.uniform(-1.0, 1.0, (ny, nx))
    u[rng.random((ny, nx)) < 0.05] = 0.0
    v[rng.random((ny, nx)) < 0.05] = 0.0
    return (np.ascontiguousarray(f), np.ascontiguousarray(u), np.ascontiguousarray(v), 2 * np.pi / nx,
            2 * np.pi / ny)


def pent_system(m: int, batch: int, seed: int):
    """Diagonally dominant batched pentadiagonal systems in the interleaved layout (arrays of shape
    (m, batch), element [i, s] = row i of system s): ds, dl, d, du, dw and a right-hand side b, with the
    zero entries of cuPentBatch's convention (ds rows 0-1, dl row 0, du row m-1, dw rows m-2, m-1)."""
    rng = np.random.default_rng(900 + seed)
    ds, dl, du, dw = (rng.uniform(-1.0, 1.0, (m, batch)) for _ in range(4))
    d = rng.uniform(5.0, 8.0, (m, batch)) * np.where(rng.random((m, batch)) < 0.5, 1.0, -1.0)
    ds[:2] = 0.0
    dl[:1] = 0.0
    du[m - 1:] = 0.0
    dw[m - 2:] = 0.0
    b = rng.uniform(-1.0, 1.0, (m, batch))
    return [np.ascontiguousarray(a) for a in (ds, dl, d, du, dw, b)]


def pent_dense_apply(ds, dl, d, du, dw, x):
    """A x for the unfactored systems (same layout), for residual checks."""
    m = x.shape[0]
    y = d * x
    y[1:] += dl[1:] * x[:-1]
    y[2:] += ds[2:] * x[:-2]
    y[:-1] += du[:-1] * x[1:]
    y[:-2] += dw[:-2] * x[2:]
    return y
