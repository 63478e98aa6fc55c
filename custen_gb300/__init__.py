"""custen_gb300 -- GB300 (sm_103a) rebuild of the cuSten 2D stencil library: Python host side.

The compute path is the in-tree shared library ``libcusten_gb300.so`` (CUDA kernels + C-ABI,
``include/custen_gb300.h``). This module binds that C-ABI with ctypes and mirrors the reference's
handle API (``cuStenCreate2D*`` / ``cuStenCompute2D*`` / ``cuStenSwap2D*`` / ``cuStenDestroy2D*``,
cuSten/src/struct/cuSten_struct_functions.h and cuSten/src/kernels/stencil_kernels.h): a
:class:`Stencil` object owns one 200-byte ``cuSten_t`` handle.

There is no CPU fallback: if the shared library is missing, importing the compute API raises.
Data arguments are device-accessible addresses (ints), or objects exposing ``data_ptr()``
(torch tensors) or ``ctypes.data`` (numpy views of managed memory).
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
# CUSTEN_CHECKED=1 selects the checked build (index checks that raise device error bit 1 instead of
# faulting; build(checked=True)).
LIB_PATH = _PKG / ("libcusten_gb300_checked.so" if os.environ.get("CUSTEN_CHECKED") == "1" else "libcusten_gb300.so")

# Variant codes (include/custen_gb300.h).
XP, XNP, XPFUN, XNPFUN, YP, YNP, YPFUN, YNPFUN, XYP, XYNP, XYPFUN, XYNPFUN = range(12)
VARIANT_NAMES = ["Xp", "Xnp", "XpFun", "XnpFun", "Yp", "Ynp", "YpFun", "YnpFun", "XYp", "XYnp", "XYpFun",
                 "XYnpFun"]
XYWENOADVP = 12   # WENO5 advection, periodic (WenoAdvection)
F64, F32 = 0, 1
DEVICE, HOST = 0, 1
HANDLE_BYTES = 200
NUM_CONFIGS = 6   # kernel configurations per element type (stencil_configs.h)

_lib = None


class CustenError(RuntimeError):
    pass


def build(checked: bool = False) -> Path:
    from . import buildlib
    return buildlib.build(checked=checked)


def lib() -> ctypes.CDLL:
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise CustenError(f"{LIB_PATH} is missing: run custen_gb300.build() (no CPU fallback exists)")
        L = ctypes.CDLL(str(LIB_PATH))
        vp, i, ull, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_size_t
        L.custen_last_error.restype = ctypes.c_char_p
        L.custen_kernel_launches.restype = ull
        L.custen_kernel_launches_tma.restype = ull
        L.custen_transfer_bytes.argtypes = [ctypes.POINTER(ull), ctypes.POINTER(ull)]
        L.custen_transfer_bytes.restype = None
        L.custen_set_stage_chunk_bytes.argtypes = [sz]
        L.custen_set_stage_chunk_bytes.restype = None
        L.custen_set_autotune.argtypes = [i]
        L.custen_set_autotune.restype = None
        L.custen_set_tune_cache.argtypes = [ctypes.c_char_p]
        L.custen_set_tune_cache.restype = None
        L.custen_tune_cache_path.argtypes = [ctypes.c_char_p, sz]
        L.custen_autotune.argtypes = [vp, i]
        L.custen_handle_config.argtypes = [vp, ctypes.c_char_p, sz]
        L.custen_set_config.argtypes = [vp, i]
        L.custen_set_fun_fusion.argtypes = [i]
        L.custen_set_fun_fusion.restype = None
        L.custen_set_max_ctas.argtypes = [i]
        L.custen_set_max_ctas.restype = None
        L.custen_builtin_fun_id.argtypes = [vp, i]
        L.custen_device_error.argtypes = [ctypes.POINTER(ctypes.c_uint), i]
        L.custen_create.argtypes = [vp, i, i, i, i, i, i, i, i, vp, vp, vp, i, i, i, i, i, i, i, vp]
        L.custen_compute_group.argtypes = [ctypes.POINTER(ctypes.c_void_p), i, i, vp]
        L.custen_create_slab.argtypes = [vp, i, i, i, i, i, i, i, i, i, vp, vp, vp, vp, vp, i, i, i, i, i, i, i, vp]
        L.custen_create_2d_xyweno_adv_p.argtypes = [vp, i, i, i, i, i, i, ctypes.c_double, ctypes.c_double, vp, vp,
                                                    vp, vp]
        L.custen_compute.argtypes = [vp, i]
        L.custen_compute_on_stream.argtypes = [vp, i, vp]
        L.custen_swap.argtypes = [vp, vp]
        L.custen_destroy.argtypes = [vp]
        L.custen_set_stream.argtypes = [vp, vp]
        L.custen_handle_variant.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(i)]
        L.custen_builtin_function.argtypes = [i, i, ctypes.POINTER(vp)]
        for name in ("custen_malloc_managed", "custen_malloc_device", "custen_malloc_host"):
            getattr(L, name).argtypes = [ctypes.POINTER(vp), sz]
        L.custen_free.argtypes = [vp]
        L.custen_free_host.argtypes = [vp]
        L.custen_memcpy.argtypes = [vp, vp, sz]
        L.custen_memset.argtypes = [vp, i, sz]
        L.custen_set_device.argtypes = [i]
        L.custen_probe_fma_rate.argtypes = [i, ctypes.POINTER(ctypes.c_double)]
        dp = ctypes.POINTER(ctypes.c_double)
        L.custen_pent_last_error.restype = ctypes.c_char_p
        for name in ("custen_pent_factor_batch",):
            getattr(L, name).argtypes = [vp, vp, vp, vp, vp, i, i, vp]
        for name in ("custen_pent_solve_batch", "custen_pent_solve_batch_rcp"):
            getattr(L, name).argtypes = [vp, vp, vp, vp, vp, vp, i, i, vp]
        L.custen_pent_invert_pivots.argtypes = [vp, i, i, vp]
        L.custen_pent_set_depth.argtypes = [i, i]
        L.custen_ch_last_error.restype = ctypes.c_char_p
        L.custen_ch_batch_create.argtypes = [ctypes.POINTER(vp), i, ctypes.POINTER(i), dp, ctypes.c_double,
                                             ctypes.c_double, i, vp]
        L.custen_ch_batch_set_state.argtypes = [vp, i, vp, vp]
        L.custen_ch_batch_get_state.argtypes = [vp, i, vp, vp]
        L.custen_ch_batch_step.argtypes = [vp, i, i]
        L.custen_ch_batch_synchronize.argtypes = [vp]
        L.custen_ch_batch_mean.argtypes = [vp, i, dp]
        L.custen_ch_batch_launches.argtypes = [vp]
        L.custen_ch_batch_launches.restype = ull
        L.custen_ch_batch_destroy.argtypes = [vp]
        L.custen_ch_batch_autotune.argtypes = [vp, i, ctypes.c_char_p, sz]
        L.custen_ch_batch_config.argtypes = [vp, ctypes.c_char_p, sz]
        L.custen_ch_batch_set_config.argtypes = [vp, i]
        L.custen_ch_batch_save.argtypes = [vp, i, ctypes.c_char_p, ctypes.c_double]
        L.custen_ch_batch_load.argtypes = [vp, i, ctypes.c_char_p, dp]
        L.custen_h5_write.argtypes = [ctypes.c_char_p, i, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(vp),
                                      ctypes.POINTER(ctypes.c_longlong)]
        L.custen_h5_read.argtypes = [ctypes.c_char_p, ctypes.c_char_p, vp, ctypes.c_longlong,
                                     ctypes.POINTER(ctypes.c_longlong)]
        L.custen_h5_last_error.restype = ctypes.c_char_p
        L.custen_ch_server_last_error.restype = ctypes.c_char_p
        L.custen_ch_server_create.argtypes = [ctypes.POINTER(vp), ctypes.c_double, i, ctypes.c_double, ctypes.c_double,
                                              i, i]
        L.custen_ch_server_submit.argtypes = [vp, i, ctypes.c_double, i, vp, ull, ctypes.c_double, ctypes.POINTER(i)]
        L.custen_ch_server_run.argtypes = [vp]
        L.custen_ch_server_result.argtypes = [vp, i, vp, dp, dp, dp, dp, dp]
        L.custen_ch_server_stats.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_longlong), dp, ctypes.POINTER(i), dp,
                                             ctypes.POINTER(ull)]
        L.custen_ch_server_destroy.argtypes = [vp]
        L.custen_ch_server_request_state.argtypes = [vp, i, ctypes.POINTER(i)]
        L.custen_ch_server_inject_failure.argtypes = [vp, i, i]
        L.custen_ch_server_set_snapshots.argtypes = [vp, i, i, ctypes.c_char_p]
        L.custen_ch_server_submit_snapshot.argtypes = [vp, ctypes.c_char_p, ctypes.c_double, i, ctypes.c_double,
                                                       ctypes.POINTER(i)]
        L.custen_ch_server_snapshots_written.argtypes = [vp, i, ctypes.POINTER(i)]
        L.custen_ch_step_noalloc.argtypes = [vp, vp, vp, i, ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]
        _lib = L
    return _lib


def _check(status: int) -> None:
    if status != 0:
        raise CustenError(lib().custen_last_error().decode(errors="replace"))


def addr(x) -> int | None:
    """Device-accessible address of x (int, torch tensor, numpy array, ctypes object or None)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if hasattr(x, "ctypes"):
        return int(x.ctypes.data)
    if isinstance(x, ctypes.c_void_p):
        return x.value
    raise TypeError(f"cannot take the address of {type(x)}")


def builtin_function(fid: int, dtype: int = F64) -> int:
    """Device address of one of the shipped Fun device functions (include/custen_gb300.h)."""
    p = ctypes.c_void_p()
    _check(lib().custen_builtin_function(fid, dtype, ctypes.byref(p)))
    return int(p.value)


def probe_fma_rate(dtype: int = F64) -> float:
    """Measured FMA/s of this GPU (all SMs, independent chains)."""
    r = ctypes.c_double()
    _check(lib().custen_probe_fma_rate(dtype, ctypes.byref(r)))
    return float(r.value)


def kernel_launches() -> int:
    return int(lib().custen_kernel_launches())


def kernel_launches_tma() -> int:
    return int(lib().custen_kernel_launches_tma())


def transfer_bytes() -> tuple:
    """(host->device, device->host) bytes moved by Compute since the library was loaded."""
    h2d, d2h = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    lib().custen_transfer_bytes(ctypes.byref(h2d), ctypes.byref(d2h))
    return int(h2d.value), int(d2h.value)


def set_autotune(mode: int) -> None:
    """0: cached configurations only (default); 1: tune launch geometries missing from the cache at a
    handle's first Compute; 2: always tune."""
    lib().custen_set_autotune(int(mode))


def set_tune_cache(path) -> None:
    """JSON file of tuned configurations (None: CUSTEN_TUNE_CACHE or ~/.cache/custen_gb300/tune.json)."""
    lib().custen_set_tune_cache(None if path is None else str(path).encode())


def tune_cache_path() -> str:
    buf = ctypes.create_string_buffer(4096)
    _check(lib().custen_tune_cache_path(buf, 4096))
    return buf.value.decode()


def set_fun_fusion(enable: bool) -> None:
    """Fused path for the library's own c^3 - c Fun functions (default on); off = indirect calls."""
    lib().custen_set_fun_fusion(int(bool(enable)))


def compute_group(stencils, offload: int = 0, stream=None) -> None:
    """One Compute of each of several independent handles (custen_compute_group), free to overlap on the
    GPU; ordered after the work queued on `stream` (a torch stream, a raw handle or None) and before work
    queued there later."""
    arr = (ctypes.c_void_p * len(stencils))(*[ctypes.addressof(st.handle) for st in stencils])
    s = 0 if stream is None else (stream if isinstance(stream, int) else int(stream.cuda_stream))
    _check(lib().custen_compute_group(arr, len(stencils), offload, s))


def set_max_ctas(max_ctas: int) -> None:
    """Cap the CTAs of a persistent stencil launch (0: no cap). Results do not depend on it."""
    lib().custen_set_max_ctas(int(max_ctas))


def set_stage_chunk_bytes(nbytes: int) -> None:
    """Chunk size for streaming host-resident fields through the GPU (0: default 32 MiB)."""
    lib().custen_set_stage_chunk_bytes(int(nbytes))


def device_error(clear: bool = True) -> int:
    """Device-side error flags (bit 0: a bounded mbarrier wait expired; bit 1, checked builds only: an
    index outside its extent, the access skipped)."""
    f = ctypes.c_uint()
    _check(lib().custen_device_error(ctypes.byref(f), int(clear)))
    return int(f.value)


def selftest_wait_expiry(rounds: int = 1 << 12) -> int:
    """Run the bounded-wait self-test (a wait nothing completes, `rounds` try_wait rounds); returns the
    device error flags seen afterwards (bit 0 expected, left set)."""
    f = ctypes.c_uint()
    st = lib().custen_selftest_wait_expiry(ctypes.c_longlong(rounds), ctypes.byref(f))
    if st != 0:
        raise CustenError(f"wait-expiry self-test failed to run (status {st})")
    return int(f.value)


class Stencil:
    """One cuSten handle. Mirrors cuStenCreate2D<variant> / Compute / Swap / Destroy.

    Window geometry: H/L/R in x, V/T/B in y (X variants: V=1, T=B=0; Y variants: H=1, L=R=0).
    ``ncoef`` defaults to the number the reference reads per Compute for the variant.
    """

    def __init__(self, variant: int, nx: int, ny: int, out, inp, coef, *, H=1, L=0, R=0, V=1, T=0, B=0,
                 num_tiles=1, block_x=32, block_y=8, dtype=F64, device=0, ncoef=None, func=None):
        self.variant, self.dtype = variant, dtype
        self.nx, self.ny = nx, ny
        self.handle = ctypes.create_string_buffer(HANDLE_BYTES)
        if ncoef is None:
            ncoef = H * V
        self._alive = False
        _check(lib().custen_create(self.handle, variant, dtype, device, num_tiles, nx, ny, block_x, block_y,
                                   addr(out), addr(inp), addr(coef), H, L, R, V, T, B, ncoef, addr(func)))
        self._alive = True

    def compute(self, offload: int = DEVICE, stream=None) -> None:
        if stream is None:
            _check(lib().custen_compute(self.handle, offload))
        else:
            s = stream if isinstance(stream, int) else int(getattr(stream, "cuda_stream", 0))
            _check(lib().custen_compute_on_stream(self.handle, offload, s))

    def swap(self, new_input) -> None:
        _check(lib().custen_swap(self.handle, addr(new_input)))

    def set_stream(self, stream) -> None:
        s = stream if (stream is None or isinstance(stream, int)) else int(stream.cuda_stream)
        _check(lib().custen_set_stream(self.handle, s))

    def destroy(self) -> None:
        if self._alive:
            self._alive = False
            _check(lib().custen_destroy(self.handle))

    def autotune(self, reps: int = 3) -> str:
        """Time every kernel configuration on this handle's launch now, cache the fastest, use it."""
        _check(lib().custen_autotune(self.handle, reps))
        return self.config()

    def set_config(self, index: int) -> None:
        """Pin this handle to kernel configuration `index` (-1: choose again at the next Compute)."""
        _check(lib().custen_set_config(self.handle, int(index)))

    def config(self) -> str:
        """Name of the kernel configuration this handle uses."""
        buf = ctypes.create_string_buffer(64)
        _check(lib().custen_handle_config(self.handle, buf, 64))
        return buf.value.decode()

    def field(self, name: str):
        """Read a cuSten_t field by name (layout of cuSten/src/struct/cuSten_struct_type.h:84-122)."""
        return getattr(CuStenT.from_buffer(self.handle), name)

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class WenoAdvection(Stencil):
    """cuStenCreate2DXYWENOADVp / Compute / Swap / Destroy: out = u * WENO5_x(in) + v * WENO5_y(in) on a
    periodic grid with spacings dx, dy (cuSten_struct_functions.h:290-347)."""

    def __init__(self, nx: int, ny: int, out, inp, u, v, *, dx: float, dy: float, num_tiles=1, block_x=32,
                 block_y=8, device=0):
        self.variant, self.dtype = XYWENOADVP, F64
        self.nx, self.ny = nx, ny
        self.handle = ctypes.create_string_buffer(HANDLE_BYTES)
        self._alive = False
        _check(lib().custen_create_2d_xyweno_adv_p(self.handle, device, num_tiles, nx, ny, block_x, block_y,
                                                   float(dx), float(dy), addr(u), addr(v), addr(out), addr(inp)))
        self._alive = True


def _pent_check(status: int) -> None:
    if status != 0:
        raise CustenError(lib().custen_pent_last_error().decode())


def pent_factor_batch(ds, dl, d, du, dw, m: int, batch: int, stream=None) -> None:
    """cuPentBatch's pentFactorBatch in place on device arrays in the interleaved layout [i * batch + s]."""
    _pent_check(lib().custen_pent_factor_batch(addr(ds), addr(dl), addr(d), addr(du), addr(dw), m, batch,
                                               _stream_ptr(stream)))


def pent_solve_batch(ds, dl, d, du, dw, b, m: int, batch: int, stream=None, inverted_pivots: bool = False) -> None:
    """cuPentBatch's pentSolveBatch (b overwritten by x); inverted_pivots: d holds 1 / pivot."""
    fn = lib().custen_pent_solve_batch_rcp if inverted_pivots else lib().custen_pent_solve_batch
    _pent_check(fn(addr(ds), addr(dl), addr(d), addr(du), addr(dw), addr(b), m, batch, _stream_ptr(stream)))


def pent_invert_pivots(d, m: int, batch: int, stream=None) -> None:
    _pent_check(lib().custen_pent_invert_pivots(addr(d), m, batch, _stream_ptr(stream)))


def _stream_ptr(stream):
    if stream is None:
        return None
    return stream if isinstance(stream, int) else int(getattr(stream, "cuda_stream", 0))


class CuStenT(ctypes.Structure):
    """ctypes view of cuSten_t (cuSten/src/struct/cuSten_struct_type.h:84-122)."""
    _fields_ = [(n, ctypes.c_int) for n in (
        "deviceNum", "numStreams", "numTiles", "nx", "ny", "nyTile", "numSten", "numStenLeft", "numStenRight",
        "numStenTop", "numStenBottom", "numStenHoriz", "numStenVert", "BLOCK_X", "BLOCK_Y", "xGrid", "yGrid",
        "mem_shared")] + [
        ("dataInput", ctypes.c_void_p), ("dataOutput", ctypes.c_void_p), ("uVel", ctypes.c_void_p),
        ("vVel", ctypes.c_void_p), ("weights", ctypes.c_void_p), ("coe", ctypes.c_void_p),
        ("coeDx", ctypes.c_double), ("coeDy", ctypes.c_double), ("numCoe", ctypes.c_int), ("nxLocal", ctypes.c_int),
        ("nyLocal", ctypes.c_int), ("boundaryTop", ctypes.c_void_p), ("boundaryBottom", ctypes.c_void_p),
        ("numBoundaryTop", ctypes.c_int), ("numBoundaryBottom", ctypes.c_int), ("streams", ctypes.c_void_p),
        ("events", ctypes.c_void_p), ("devFunc", ctypes.c_void_p)]


assert ctypes.sizeof(CuStenT) == HANDLE_BYTES


def create_reference_style(variant: int, nx: int, ny: int, out, inp, coef, *, num_sten=None, L=0, R=0, T=0, B=0,
                           H=None, V=None, num_tiles=1, block_x=32, block_y=8, num_coe=None, func=None,
                           dtype=F64, device=0) -> Stencil:
    """Create a handle from the reference's per-variant argument meaning (numSten / numCoe)."""
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    fun = variant in (XPFUN, XNPFUN, YPFUN, YNPFUN, XYPFUN, XYNPFUN)
    if d == 0:
        Hh, Vv = (L + R + 1 if fun else num_sten), 1
        ncoef = num_coe if fun else num_sten
    elif d == 1:
        Hh, Vv = 1, (T + B + 1 if fun else num_sten)
        ncoef = (num_coe if variant == YPFUN else num_sten) if fun else num_sten
    else:
        Hh, Vv = H, V
        ncoef = H * V
    return Stencil(variant, nx, ny, out, inp, coef, H=Hh, L=L, R=R, V=Vv, T=T, B=B, num_tiles=num_tiles,
                   block_x=block_x, block_y=block_y, dtype=dtype, device=device, ncoef=ncoef, func=func)


def _ch_check(status: int) -> None:
    if status != 0:
        raise CustenError(lib().custen_ch_last_error().decode(errors="replace"))


def snapshot_name(time: float) -> str:
    """File name of the reference solver's snapshot at `time` (cuPentCahnADI.cu:107-110)."""
    return "cahn_hilliard_%0.10f.nc" % time


def h5_write(path, datasets) -> None:
    """Write an HDF5 file whose root group holds the given two-dimensional float64 datasets
    ({name: array}, 1 to 8 of them), in the format of the reference solver's snapshots."""
    import numpy as np
    items = [(str(k), np.ascontiguousarray(v, dtype=np.float64)) for k, v in dict(datasets).items()]
    arrays = [a.reshape(a.shape if a.ndim == 2 else (a.size, 1) if a.ndim == 1 else (1, 1)) for _, a in items]
    if any(a.ndim != 2 for a in arrays):
        raise CustenError("h5_write: datasets must have rank 0, 1 or 2")
    names = (ctypes.c_char_p * len(items))(*[k.encode() for k, _ in items])
    ptrs = (ctypes.c_void_p * len(items))(*[a.ctypes.data for a in arrays])
    dims = (ctypes.c_longlong * (2 * len(items)))(*[d for a in arrays for d in a.shape])
    if lib().custen_h5_write(os.fsencode(path), len(items), names, ptrs, dims) != 0:
        raise CustenError(lib().custen_h5_last_error().decode(errors="replace"))


def h5_read(path, name: str):
    """Read one float dataset of an HDF5 file (version-0/1 superblock, contiguous storage) as a
    two-dimensional float64 array."""
    import numpy as np
    dims = (ctypes.c_longlong * 2)()
    L = lib()
    if L.custen_h5_read(os.fsencode(path), name.encode(), None, 0, dims) != 0:
        raise CustenError(L.custen_h5_last_error().decode(errors="replace"))
    out = np.empty((dims[0], dims[1]))
    if L.custen_h5_read(os.fsencode(path), name.encode(), out.ctypes.data, out.size, dims) != 0:
        raise CustenError(L.custen_h5_last_error().decode(errors="replace"))
    return out


class CahnHilliardBatch:
    """Many periodic Cahn-Hilliard ADI simulations of different sizes advanced together on the GPU
    (the solver of cuPentCahnADI, batched; include/custen_gb300.h)."""

    def __init__(self, sizes, lx=None, gamma: float = 0.01, dt_factor: float = 0.1, rhs_dtype: int = F64,
                 stream=None):
        import numpy as np
        self.sizes = [int(n) for n in sizes]
        ns = (ctypes.c_int * len(self.sizes))(*self.sizes)
        lxa = None
        if lx is not None:
            lxv = [float(v) for v in (lx if hasattr(lx, "__len__") else [lx] * len(self.sizes))]
            lxa = (ctypes.c_double * len(lxv))(*lxv)
        h = ctypes.c_void_p()
        s = stream if (stream is None or isinstance(stream, int)) else int(stream.cuda_stream)
        _ch_check(lib().custen_ch_batch_create(ctypes.byref(h), len(self.sizes), ns, lxa, gamma, dt_factor, rhs_dtype,
                                               s))
        self.h = h.value
        self._np = np

    def set_state(self, sim: int, c_cur, c_old=None) -> None:
        np = self._np
        n = self.sizes[sim]
        c_cur = np.ascontiguousarray(c_cur, dtype=np.float64).reshape(n, n)
        c_old = None if c_old is None else np.ascontiguousarray(c_old, dtype=np.float64).reshape(n, n)
        _ch_check(lib().custen_ch_batch_set_state(self.h, sim, c_cur.ctypes.data,
                                                  None if c_old is None else c_old.ctypes.data))

    def state(self, sim: int):
        np = self._np
        n = self.sizes[sim]
        cur, old = np.empty((n, n)), np.empty((n, n))
        _ch_check(lib().custen_ch_batch_get_state(self.h, sim, cur.ctypes.data, old.ctypes.data))
        return cur, old

    def step(self, steps: int = 1, graph: bool = True) -> None:
        _ch_check(lib().custen_ch_batch_step(self.h, steps, int(graph)))

    def autotune(self, steps: int = 4) -> str:
        """Time every kernel configuration on this batch (state restored afterwards); keep the fastest."""
        buf = ctypes.create_string_buffer(64)
        _ch_check(lib().custen_ch_batch_autotune(self.h, int(steps), buf, 64))
        return buf.value.decode()

    def config(self) -> str:
        buf = ctypes.create_string_buffer(64)
        _ch_check(lib().custen_ch_batch_config(self.h, buf, 64))
        return buf.value.decode()

    def set_config(self, index: int) -> None:
        """Pin the kernel configuration (0 .. 21; -1: the default)."""
        _ch_check(lib().custen_ch_batch_set_config(self.h, int(index)))

    def save(self, sim: int, path, time: float = 0.0) -> None:
        """Write grid `sim` to an HDF5 snapshot: "c" (cCurr, the reference's dataset), "c_old", "t"."""
        _ch_check(lib().custen_ch_batch_save(self.h, sim, os.fsencode(path), float(time)))

    def load(self, sim: int, path) -> float:
        """Resume grid `sim` from an HDF5 snapshot (this library's or the reference's); returns its time
        (NaN when the file has none)."""
        t = ctypes.c_double()
        _ch_check(lib().custen_ch_batch_load(self.h, sim, os.fsencode(path), ctypes.byref(t)))
        return float(t.value)

    def synchronize(self) -> None:
        _ch_check(lib().custen_ch_batch_synchronize(self.h))

    def mean(self, sim: int) -> float:
        m = ctypes.c_double()
        _ch_check(lib().custen_ch_batch_mean(self.h, sim, ctypes.byref(m)))
        return float(m.value)

    def launches(self) -> int:
        return int(lib().custen_ch_batch_launches(self.h))

    def close(self) -> None:
        if self.h:
            lib().custen_ch_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _srv_check(status: int) -> None:
    if status != 0:
        raise CustenError(lib().custen_ch_server_last_error().decode(errors="replace"))


class CahnHilliardServer:
    """Request loop with continuous batching of Cahn-Hilliard simulations (include/custen_gb300.h)."""

    def __init__(self, hbm_budget_bytes: float = 150e9, rhs_dtype: int = F64, gamma: float = 0.01,
                 dt_factor: float = 0.1, chunk_steps: int = 8, keep_results: bool = True):
        h = ctypes.c_void_p()
        _srv_check(lib().custen_ch_server_create(ctypes.byref(h), hbm_budget_bytes, rhs_dtype, gamma, dt_factor,
                                                 chunk_steps, int(keep_results)))
        self.h = h.value
        self.sizes = []

    def submit(self, n: int, steps: int, arrival: float = 0.0, c0=None, seed: int = 0, lx: float = 0.0) -> int:
        import numpy as np
        rid = ctypes.c_int()
        ptr = None
        if c0 is not None:
            c0 = np.ascontiguousarray(c0, dtype=np.float64)
            ptr = c0.ctypes.data
        _srv_check(lib().custen_ch_server_submit(self.h, n, lx, steps, ptr, seed, arrival, ctypes.byref(rid)))
        self.sizes.append(n)
        return rid.value

    def run(self) -> None:
        _srv_check(lib().custen_ch_server_run(self.h))

    def result(self, rid: int, field: bool = True):
        import numpy as np
        n = self.sizes[rid]
        out = np.empty((n, n)) if field else None
        vals = [ctypes.c_double() for _ in range(5)]
        _srv_check(lib().custen_ch_server_result(self.h, rid, None if out is None else out.ctypes.data,
                                                 *[ctypes.byref(v) for v in vals]))
        arrival, admit, done, m0, m1 = (v.value for v in vals)
        return {"field": out, "arrival": arrival, "admit": admit, "done": done, "mean0": m0, "mean_end": m1,
                "ttc": done - arrival}

    def state(self, rid: int) -> str:
        """"pending", "resident", "done" or "failed" (result() then raises with the reason)."""
        st = ctypes.c_int()
        _srv_check(lib().custen_ch_server_request_state(self.h, rid, ctypes.byref(st)))
        return ("pending", "resident", "done", "failed")[st.value]

    def snapshots(self, rid: int, every: int, directory) -> None:
        """Write the request's state every `every` steps to directory/cahn_hilliard_<time>.nc."""
        _srv_check(lib().custen_ch_server_set_snapshots(self.h, rid, int(every), os.fsencode(directory)))

    def snapshots_written(self, rid: int) -> int:
        c = ctypes.c_int()
        _srv_check(lib().custen_ch_server_snapshots_written(self.h, rid, ctypes.byref(c)))
        return c.value

    def submit_snapshot(self, path, steps: int, arrival: float = 0.0, lx: float = 0.0) -> int:
        """Queue a request resumed from a snapshot file; it advances `steps` more steps."""
        rid = ctypes.c_int()
        _srv_check(lib().custen_ch_server_submit_snapshot(self.h, os.fsencode(path), lx, steps, arrival,
                                                          ctypes.byref(rid)))
        dims = (ctypes.c_longlong * 2)()
        lib().custen_h5_read(os.fsencode(path), b"c", None, 0, dims)
        self.sizes.append(int(dims[0]))
        return rid.value

    def inject_failure(self, rid: int, kind: int = 1) -> None:
        """Test hook: make the request's admission allocation fail (kind 1), on the host."""
        _srv_check(lib().custen_ch_server_inject_failure(self.h, rid, kind))

    def stats(self):
        mk, pts, bts = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        st, ma, la = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_ulonglong()
        _srv_check(lib().custen_ch_server_stats(self.h, ctypes.byref(mk), ctypes.byref(st), ctypes.byref(pts),
                                                ctypes.byref(ma), ctypes.byref(bts), ctypes.byref(la)))
        return {"makespan": mk.value, "steps": st.value, "point_steps": pts.value, "max_active": ma.value,
                "peak_bytes": bts.value, "launches": la.value}

    def close(self):
        if self.h:
            lib().custen_ch_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
