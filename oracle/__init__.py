"""Oracles -- TEST INFRASTRUCTURE ONLY (used by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg as the checker; never by the library).

* ``stencil_oracle.c``: C restatement of the twelve cuSten stencil kernels (block-by-block emulation,
  see the header of that file).
* ``weno_oracle.c``: C restatement of the periodic WENO5 advection operator
  (cuSten/src/kernels/2d_xyADVWENO_p_kernel.cu).
* ``pent_oracle.c``: C restatement of cuPentBatch's batched pentadiagonal factorisation and solve.
* ``ch_oracle.c``: C restatement of the Cahn-Hilliard ADI solver of
  cuPentSpeedUp/serialCahnADITiming/serialCahnADI.c.
* ``ref_build.py``: builds the reference's own code from the reference sources into ``oracle/_ref``
  (the serial Cahn-Hilliard program as a shared library, and the cuSten kernels as an sm_103a cubin);
  only possible where the reference sources are present.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SOURCES = [HERE / "stencil_oracle.c", HERE / "ch_oracle.c", HERE / "weno_oracle.c", HERE / "pent_oracle.c"]
HEADERS = [HERE / "stencil_oracle_impl.h"]

REFRUN = BUILD / "librefrun.so"
REFCH = BUILD / "librefch.so"
REF_CUBIN = HERE / "_ref" / "custen_ref_sm103a.cubin"
REF_CH_CUBIN = HERE / "_ref" / "custen_ref_ch_sm103a.cubin"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))

_lib = None
_refrun = None


def _build_refrun() -> None:
    src = HERE / "ref_runner.cpp"
    if REFRUN.exists() and REFRUN.stat().st_mtime >= src.stat().st_mtime:
        return
    tmp = REFRUN.with_suffix(".so.tmp")
    libdirs = [CUDA_HOME / "lib64", CUDA_HOME / "lib64" / "stubs", CUDA_HOME / "targets" / "sbsa-linux" / "lib" / "stubs"]
    cmd = ["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-I", str(CUDA_HOME / "include"), "-o", str(tmp), str(src)]
    for d in libdirs:
        if d.exists():
            cmd += ["-L", str(d)]
    cmd += ["-lcuda"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REFRUN)


def _build_refch() -> None:
    src = HERE / "ref_ch_runner.cpp"
    if REFCH.exists() and REFCH.stat().st_mtime >= src.stat().st_mtime:
        return
    tmp = REFCH.with_suffix(".so.tmp")
    libdirs = [CUDA_HOME / "lib64", CUDA_HOME / "lib64" / "stubs", CUDA_HOME / "targets" / "sbsa-linux" / "lib",
               CUDA_HOME / "targets" / "sbsa-linux" / "lib" / "stubs"]
    # contraction off: the program's host-side coefficients are plain IEEE expressions
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17", "-I", str(CUDA_HOME / "include"),
           "-o", str(tmp), str(src)]
    for d in libdirs:
        if d.exists():
            cmd += ["-L", str(d)]
    cmd += ["-lcublas", "-lcudart", "-lcuda"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REFCH)


def build() -> Path:
    """Compile the C oracles (gcc, contraction off so that every fma is explicit)."""
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = [s for s in SOURCES if s.exists()]
    deps = srcs + HEADERS
    if not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-o", str(tmp),
               *map(str, srcs), "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    _build_refrun()
    _build_refch()
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        vp, i = ctypes.c_void_p, ctypes.c_int
        for name in ("oracle_stencil_f64", "oracle_stencil_f32"):
            f = getattr(L, name)
            f.argtypes = [i, i, i, i, i, i, vp, vp, vp, vp, i, i, i, i, i, i, i, i, vp]
            f.restype = i
        L.oracle_host_loop_xyp_f64.argtypes = [i, i, vp, vp, vp, i, i, i, i, i, i]
        L.oracle_host_loop_f64.argtypes = [i, i, vp, vp, vp, i, i, i, i, i, i, i]
        L.oracle_weno_f64.argtypes = [i, i, vp, vp, vp, vp, ctypes.c_double, ctypes.c_double]
        L.oracle_weno_f64.restype = None
        L.oracle_pent_factor.argtypes = [vp, vp, vp, vp, vp, i, i]
        L.oracle_pent_factor.restype = None
        L.oracle_pent_solve.argtypes = [vp, vp, vp, vp, vp, vp, i, i]
        L.oracle_pent_solve.restype = None
        L.ch_oracle_create.argtypes = [i, ctypes.c_double, vp]
        L.ch_oracle_create.restype = vp
        L.ch_oracle_step.argtypes = [vp, i]
        L.ch_oracle_get.argtypes = [vp, vp, vp]
        L.ch_oracle_tables.argtypes = [vp, vp]
        L.ch_oracle_destroy.argtypes = [vp]
        L.ch_oracle_mean.argtypes = [vp, ctypes.c_longlong]
        L.ch_oracle_mean.restype = ctypes.c_double
        _lib = L
    return _lib


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def stencil(variant: int, out: np.ndarray, inp: np.ndarray, coef: np.ndarray, *, num_tiles: int, block_x: int,
            block_y: int, H: int, L: int, R: int, V: int, T: int, B: int, fun_id: int = -1,
            halo_src: np.ndarray | None = None) -> np.ndarray:
    """One Compute of `variant`; `out` (ny x nx) is updated in place. Returns the status array
    (0 untouched, 1 written, 2 written from shared memory the reference never loaded)."""
    assert out.dtype == inp.dtype == coef.dtype and out.flags.c_contiguous and inp.flags.c_contiguous
    ny, nx = inp.shape
    status = np.zeros((ny, nx), dtype=np.uint8)
    fn = lib().oracle_stencil_f64 if inp.dtype == np.float64 else lib().oracle_stencil_f32
    coef = np.ascontiguousarray(coef)
    rc = fn(variant, nx, ny, num_tiles, block_x, block_y, _p(out), _p(inp), _p(halo_src), _p(coef), coef.size, H, L,
            R, V, T, B, fun_id, _p(status))
    if rc != 0:
        raise ValueError("configuration outside the reference kernels' contract")
    return status


def weno(inp: np.ndarray, u: np.ndarray, v: np.ndarray, cdx: float, cdy: float) -> np.ndarray:
    """Periodic WENO5 advection, out = u * Fx + v * Fy (weno_oracle.c); cdx = 1/dx, cdy = 1/dy."""
    inp, u, v = (np.ascontiguousarray(a, dtype=np.float64) for a in (inp, u, v))
    ny, nx = inp.shape
    out = np.empty_like(inp)
    lib().oracle_weno_f64(nx, ny, inp.ctypes.data, u.ctypes.data, v.ctypes.data, out.ctypes.data, float(cdx),
                          float(cdy))
    return out


def pent_factor(ds, dl, d, du, dw):
    """cuPentBatch's pentFactorBatch on (m, batch) arrays in the interleaved layout; returns new arrays."""
    arrs = [np.array(a, dtype=np.float64, order="C", copy=True) for a in (ds, dl, d, du, dw)]
    m, batch = arrs[0].shape
    lib().oracle_pent_factor(*[a.ctypes.data for a in arrs], m, batch)
    return arrs


def pent_solve(factors, b):
    """cuPentBatch's pentSolveBatch with the factors of pent_factor; returns the solution."""
    fs = [np.ascontiguousarray(a, dtype=np.float64) for a in factors]
    x = np.array(b, dtype=np.float64, order="C", copy=True)
    m, batch = x.shape
    lib().oracle_pent_solve(*[a.ctypes.data for a in fs], x.ctypes.data, m, batch)
    return x


def host_loop_xyp(inp: np.ndarray, w: np.ndarray, H: int, L: int, V: int, T: int, y0: int = 0,
                  y1: int | None = None) -> np.ndarray:
    """Plain periodic host loop (CPU baseline), rows [y0, y1)."""
    ny, nx = inp.shape
    out = np.zeros_like(inp)
    w = np.ascontiguousarray(w, dtype=np.float64)
    lib().oracle_host_loop_xyp_f64(nx, ny, _p(inp), _p(out), _p(w), H, L, V, T, y0, ny if y1 is None else y1)
    return out


def host_loop(inp: np.ndarray, out: np.ndarray, w: np.ndarray, H: int, L: int, V: int, T: int, cube: bool,
              y0: int, y1: int) -> None:
    """Plain periodic host loop over rows [y0, y1) into `out` (releases the GIL: callable from threads)."""
    ny, nx = inp.shape
    lib().oracle_host_loop_f64(nx, ny, _p(inp), _p(out), _p(np.ascontiguousarray(w, dtype=np.float64)), H, L, V, T,
                               int(cube), y0, y1)


class CHOracle:
    """The C restatement of the serial Cahn-Hilliard ADI solver (ch_oracle.c)."""

    def __init__(self, c0: np.ndarray, lx: float = 2 * np.pi):
        L = lib()
        n = c0.shape[0]
        assert c0.shape == (n, n)
        self.n = n
        self._c0 = np.ascontiguousarray(c0, dtype=np.float64)
        self._h = L.ch_oracle_create(n, lx, _p(self._c0))

    def step(self, steps: int = 1) -> None:
        lib().ch_oracle_step(self._h, steps)

    def fields(self):
        cur = np.empty((self.n, self.n))
        old = np.empty((self.n, self.n))
        lib().ch_oracle_get(self._h, _p(cur), _p(old))
        return cur, old

    def tables(self) -> np.ndarray:
        m = self.n - 2
        out = np.empty(7 * m + 4)
        lib().ch_oracle_tables(self._h, _p(out))
        return out

    def __del__(self):
        try:
            lib().ch_oracle_destroy(self._h)
        except Exception:
            pass


def compensated_mean(c: np.ndarray) -> float:
    c = np.ascontiguousarray(c, dtype=np.float64)
    return float(lib().ch_oracle_mean(_p(c), c.size))


SERIAL_REF = HERE / "_ref" / "libserialch.so"


def reference_serial_ch(c0: np.ndarray, steps: int, lx: float = 2 * np.pi):
    """The reference's own serialCahnADI.c functions (built from its source); None if not built."""
    if not SERIAL_REF.exists():
        return None
    R = ctypes.CDLL(str(SERIAL_REF))
    R.ref_ch_run.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.c_void_p]
    n = c0.shape[0]
    c0 = np.ascontiguousarray(c0, dtype=np.float64)
    cur, old = np.empty((n, n)), np.empty((n, n))
    R.ref_ch_run(n, lx, steps, _p(c0), _p(cur), _p(old))
    return cur, old


def reference_kernels():
    """ctypes handle on the runner of the reference's own kernels (cubin built from the reference
    sources); None when the cubin is not present."""
    global _refrun
    if _refrun is None:
        if not REF_CUBIN.exists():
            return None
        build()
        R = ctypes.CDLL(str(REFRUN))
        vp, i = ctypes.c_void_p, ctypes.c_int
        R.refrun_error.restype = ctypes.c_char_p
        R.refrun_load.argtypes = [ctypes.c_char_p]
        R.refrun_fun_ptr.argtypes = [i, ctypes.POINTER(ctypes.c_ulonglong)]
        R.refrun_compute.argtypes = [i, i, i, i, i, i, vp, vp, vp, vp, i, i, i, i, i, i, i, i, ctypes.c_ulonglong]
        R.refrun_weno.argtypes = [i, i, i, i, i, vp, vp, vp, vp, ctypes.c_double, ctypes.c_double]
        if R.refrun_load(str(REF_CUBIN).encode()) != 0:
            raise RuntimeError(R.refrun_error().decode())
        _refrun = R
    return _refrun


def reference_fun_ptr(fid: int) -> int:
    R = reference_kernels()
    p = ctypes.c_ulonglong()
    if R.refrun_fun_ptr(fid, ctypes.byref(p)) != 0:
        raise RuntimeError(R.refrun_error().decode())
    return int(p.value)


def reference_compute(variant: int, nx: int, ny: int, num_tiles: int, bx: int, by: int, out_ptr: int, in_ptr: int,
                      coef_ptr: int, *, num_sten: int, H: int, L: int, R: int, V: int, T: int, B: int, num_coe: int = 0,
                      func: int = 0, halo_ptr: int | None = None) -> None:
    """One Compute of the reference kernel itself on device buffers (device pointers)."""
    Rr = reference_kernels()
    rc = Rr.refrun_compute(variant, nx, ny, num_tiles, bx, by, out_ptr, in_ptr, halo_ptr or in_ptr, coef_ptr,
                           num_sten, H, L, R, V, T, B, num_coe, func)
    if rc != 0:
        raise RuntimeError(Rr.refrun_error().decode())


def reference_weno(nx: int, ny: int, num_tiles: int, bx: int, by: int, out_ptr: int, in_ptr: int, u_ptr: int,
                   v_ptr: int, cdx: float, cdy: float) -> None:
    """One Compute of the reference's WENO advection kernel on device buffers (device pointers)."""
    Rr = reference_kernels()
    rc = Rr.refrun_weno(nx, ny, num_tiles, bx, by, out_ptr, in_ptr, u_ptr, v_ptr, float(cdx), float(cdy))
    if rc != 0:
        raise RuntimeError(Rr.refrun_error().decode())


_refch = None


class ReferenceCahnHilliardGPU:
    """The reference's Cahn-Hilliard GPU program (cuPentCahnADITiming), device code unchanged, host loop
    restated in oracle/ref_ch_runner.cpp: one grid, one step at a time with its device synchronisations.
    Needs oracle/_ref/custen_ref_ch_sm103a.cubin (built where the reference sources exist)."""

    @staticmethod
    def available() -> bool:
        return REF_CH_CUBIN.exists()

    @staticmethod
    def _load():
        global _refch
        if _refch is None:
            build()
            R = ctypes.CDLL(str(REFCH))
            vp, i = ctypes.c_void_p, ctypes.c_int
            R.refch_error.restype = ctypes.c_char_p
            R.refch_load.argtypes = [ctypes.c_char_p]
            R.refch_create.argtypes = [ctypes.POINTER(vp), i, ctypes.c_double, vp, vp, vp, vp]
            R.refch_step.argtypes = [vp, i]
            R.refch_get.argtypes = [vp, vp, vp]
            R.refch_destroy.argtypes = [vp]
            R.refch_pent_factor.argtypes = [vp, vp, vp, vp, vp, i, i]
            R.refch_pent_solve.argtypes = [vp, vp, vp, vp, vp, vp, i, i]
            if R.refch_load(str(REF_CH_CUBIN).encode()) != 0:
                raise RuntimeError(R.refch_error().decode())
            _refch = R
        return _refch

    def __init__(self, c0: np.ndarray, lx: float = 2 * np.pi):
        self._R = self._load()
        c0 = np.ascontiguousarray(c0, dtype=np.float64)
        n = c0.shape[0]
        self.n = n
        tabs = CHOracle(c0, lx=lx).tables()
        m = n - 2
        inv1, inv2, omega = (np.ascontiguousarray(tabs[5 * m:6 * m]), np.ascontiguousarray(tabs[6 * m:7 * m]),
                             np.ascontiguousarray(tabs[7 * m:7 * m + 4]))
        h = ctypes.c_void_p()
        if self._R.refch_create(ctypes.byref(h), n, float(lx), c0.ctypes.data, omega.ctypes.data, inv1.ctypes.data,
                                inv2.ctypes.data) != 0:
            raise RuntimeError(self._R.refch_error().decode())
        self._h = h

    def step(self, steps: int) -> None:
        if self._R.refch_step(self._h, int(steps)) != 0:
            raise RuntimeError(self._R.refch_error().decode())

    def state(self):
        cur, old = np.empty((self.n, self.n)), np.empty((self.n, self.n))
        if self._R.refch_get(self._h, cur.ctypes.data, old.ctypes.data) != 0:
            raise RuntimeError(self._R.refch_error().decode())
        return cur, old

    def close(self) -> None:
        if self._h:
            self._R.refch_destroy(self._h)
            self._h = None


def reference_pent(factor: bool, ptrs, m: int, batch: int) -> None:
    """Run the reference's pentFactorBatch (ptrs: ds, dl, d, du, dw) or pentSolveBatch (ptrs: ds, dl, d,
    du, dw, b) on device pointers (the reference CH cubin)."""
    ReferenceCahnHilliardGPU._load()
    R = _refch
    rc = R.refch_pent_factor(*ptrs, m, batch) if factor else R.refch_pent_solve(*ptrs, m, batch)
    if rc != 0:
        raise RuntimeError(R.refch_error().decode())
