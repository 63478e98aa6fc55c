"""The shared library loads on a CPU-only machine and exports every symbol the headers declare:
the reference's C++ API under its exact mangled names (include/cuSten.h) and the C-ABI
(include/custen_gb300.h). No compute call is made here."""
import ctypes
import re
from pathlib import Path

import pytest

import custen_gb300 as cs

ROOT = Path(__file__).resolve().parent.parent


def _decls(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    for m in re.finditer(r"\b(void|int|unsigned long long|const char\*)\s+(\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        yield m.group(2), [a.strip() for a in m.group(3).split(",") if a.strip() and a.strip() != "void"]


def _mangle(name: str, params: list[str]) -> str:
    """Itanium C++ mangling for the argument types used by the cuSten API."""
    out, seen_pd = [], False
    for p in params:
        t = re.sub(r"\s+\w+$", "", p).replace(" ", "")
        if t == "cuSten_t*":
            out.append("P8cuSten_t")
        elif t == "int":
            out.append("i")
        elif t == "bool":
            out.append("b")
        elif t == "double":
            out.append("d")
        elif t == "constchar*":
            out.append("PKc")
        elif t == "double*":
            out.append("S1_" if seen_pd else "Pd")
            seen_pd = True
        else:
            raise AssertionError(f"unexpected parameter type {t!r} in {name}")
    return f"_Z{len(name)}{name}{''.join(out)}"


def test_library_loads(built):
    assert cs.lib().custen_sizeof_handle() == 200
    assert cs.lib().custen_abi_version() >= 1
    assert ctypes.sizeof(cs.CuStenT) == 200
    assert cs.CuStenT.weights.offset == 104 and cs.CuStenT.streams.offset == 176 and cs.CuStenT.devFunc.offset == 192


def test_cpp_dropin_symbols(built):
    L = cs.lib()
    names = list(_decls(ROOT / "include" / "cuSten.h"))
    # 13 operators x (create, swap, destroy, compute) + cuSenCompute2DXpFun + checkError
    assert len(names) == 54
    for name, params in names:
        mangled = _mangle(name, params)
        assert hasattr(L, mangled), f"missing {name} as {mangled}"
    # spot-check against names measured from the reference library build
    for m in ("_Z16cuStenCreate2DXpP8cuSten_tiiiiiiPdS1_S1_iii", "_Z17cuStenCompute2DXpP8cuSten_tb",
              "_Z14cuStenSwap2DXpP8cuSten_tPd", "_Z19cuSenCompute2DXpFunP8cuSten_tb",
              "_Z17cuStenCreate2DXYpP8cuSten_tiiiiiiPdS1_S1_iiiiii",
              "_Z24cuStenCreate2DXYWENOADVpP8cuSten_tiiiiiiddPdS1_S1_S1_"):
        assert hasattr(L, m), m


def test_c_abi_symbols(built):
    L = cs.lib()
    names = [n for n, _ in _decls(ROOT / "include" / "custen_gb300.h")]
    assert len(names) > 20
    for n in names:
        assert hasattr(L, n), f"C-ABI entry point {n} not exported"


def test_errors_are_status_codes_not_exits(built):
    """Argument errors come back as a status with a message; the process keeps running."""
    h = ctypes.create_string_buffer(200)
    rc = cs.lib().custen_create(h, cs.XP, cs.F64, 0, 3, 64, 64, 32, 8, 1, 1, 1, 5, 2, 2, 1, 0, 0, 5, None)
    assert rc == 2
    assert b"divisible by numTiles" in cs.lib().custen_last_error()
    rc = cs.lib().custen_compute(h, 0)
    assert rc == 2 and b"not created" in cs.lib().custen_last_error()


def test_group_and_slab_argument_errors(built):
    """Argument checks of custen_compute_group and custen_create_slab run before any device work."""
    L = cs.lib()
    assert L.custen_compute_group(None, 0, 0, None) == 0
    assert L.custen_compute_group(None, -1, 0, None) == 2
    stale = ctypes.create_string_buffer(200)
    arr = (ctypes.c_void_p * 1)(ctypes.addressof(stale))
    assert L.custen_compute_group(arr, 1, 0, None) == 2
    assert b"not created by this library" in L.custen_last_error()
    h = ctypes.create_string_buffer(200)
    rc = L.custen_create_slab(h, cs.YP, cs.F64, 0, 3, 2, 64, 64, 32, 8, 1, 1, 1, 1, 1, 1, 0, 0, 5, 2, 2, 5, None)
    assert rc == 2 and b"index must lie" in L.custen_last_error()
    rc = L.custen_create_slab(h, cs.YP, cs.F64, 0, 1, 2, 64, 64, 32, 8, 1, 1, None, 1, 1, 1, 0, 0, 5, 2, 2, 5, None)
    assert rc == 2 and b"halo_top is NULL" in L.custen_last_error()
