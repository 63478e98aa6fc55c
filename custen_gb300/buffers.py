"""Device, managed and pinned host allocations made through the library's C-ABI, with numpy views.

Used by the benchmark, the smoke run and the tests to hold fields without torch.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _check, lib


class DeviceBuffer:
    """Device (or managed) allocation made through the C-ABI (no torch needed)."""

    def __init__(self, nbytes: int, managed: bool = False):
        self.nbytes = nbytes
        self.managed = managed
        p = ctypes.c_void_p()
        fn = lib().custen_malloc_managed if managed else lib().custen_malloc_device
        _check(fn(ctypes.byref(p), max(nbytes, 16)))
        self.ptr = int(p.value)

    @classmethod
    def from_array(cls, a: np.ndarray, managed: bool = False) -> "DeviceBuffer":
        b = cls(a.nbytes, managed)
        b.upload(a)
        return b

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        _check(lib().custen_memcpy(self.ptr, a.ctypes.data, a.nbytes))

    def download(self, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        _check(lib().custen_memcpy(out.ctypes.data, self.ptr, out.nbytes))
        return out

    def view(self, shape, dtype) -> np.ndarray:
        """Host view of managed memory (valid after a device synchronize)."""
        assert self.managed
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        buf = (ctypes.c_char * n).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            lib().custen_free(self.ptr)
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
        _check(lib().custen_malloc_host(ctypes.byref(p), max(nbytes, 16)))
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
            lib().custen_free_host(self.ptr)
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
