"""Build recipe for the sm_103a libraries of this package.

Outputs (in-tree, git-ignored):
  custen_gb300/libcusten_gb300.so  -- shared library: C-ABI (include/custen_gb300.h), the C++ drop-in API
                                      (include/cuSten.h), kernels and the shipped Fun device functions.
  custen_gb300/libcuSten.a         -- static drop-in for the reference's libcuSten.a (relocatable device
                                      code; link the user program with nvcc -rdc=true, as with the reference).
  custen_gb300/libcusten_gb300_checked.so -- build(checked=True) only: the shared library compiled with
                                      -DCUSTEN_CHECKED=1 (index checks that raise a device error flag instead
                                      of faulting, csrc/checked.cuh); loaded when CUSTEN_CHECKED=1.

Every translation unit is compiled for sm_103a only, with relocatable device code so that the Fun
variants can call device functions defined in other translation units.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build" / "custen_gb300"
SO_PATH = PKG / "libcusten_gb300.so"
A_PATH = PKG / "libcuSten.a"
CHECKED_BUILD = ROOT / "_build" / "custen_gb300_checked"
CHECKED_SO_PATH = PKG / "libcusten_gb300_checked.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-rdc=true", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]

# stencil_cfg.cu is compiled once per entry of the configuration table (stencil_configs.h).
NUM_CONFIGS = 6
CFG_UNITS = [(f"stencil_cfg_{d}_{k}", "stencil_cfg.cu", [f"-DCUSTEN_CFG_DTYPE={d}", f"-DCUSTEN_CFG_INDEX={k}"])
             for d in (0, 1) for k in range(NUM_CONFIGS)]
# Translation units of the static drop-in library (the reference's libcuSten.a surface):
# (object name, source, extra flags).
LIB_UNITS = [("plan", "plan.cu", []), ("stencil_dispatch", "stencil_dispatch.cu", []), ("weno", "weno.cu", []),
             ("autotune", "autotune.cu", [])] + CFG_UNITS
# Extra translation units of the shared library.
SO_UNITS = [(Path(s).stem, s, []) for s in ("builtin_funs.cu", "probe.cu", "ch_solver.cu", "ch_server.cu",
                                            "pent_batch.cu", "h5snap.cpp", "selftest.cu")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}")


def _needs(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))


def build(verbose: bool = False, jobs: int | None = None, checked: bool = False) -> Path:
    build_dir = CHECKED_BUILD if checked else BUILD
    so_path = CHECKED_SO_PATH if checked else SO_PATH
    build_dir.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    units = LIB_UNITS + SO_UNITS
    objs = {name: build_dir / (name + ".o") for name, _, _ in units}
    defs = ["-DCUSTEN_CHECKED=1"] if checked else []

    def compile_one(unit) -> None:
        name, src, extra = unit
        out = objs[name]
        if _needs(out, [CSRC / src] + hdrs):
            cmd = [cc, *ARCH, *NVCC_FLAGS, *defs, *extra, "-c", str(CSRC / src), "-o", str(out)]
            if verbose:
                print(" ".join(cmd), flush=True)
            _run(cmd)

    with cf.ThreadPoolExecutor(max_workers=jobs or max(1, min(16, os.cpu_count() or 1, len(units)))) as ex:
        list(ex.map(compile_one, units))

    all_objs = [str(objs[name]) for name, _, _ in units]
    if _needs(so_path, list(objs.values())):
        tmp = so_path.with_suffix(".so.tmp")
        _run([cc, *ARCH, "-shared", "-rdc=true", "-Xcompiler", "-fPIC", *all_objs, "-o", str(tmp), "-cudart",
              "static"])
        os.replace(tmp, so_path)
    if checked:
        return so_path
    lib_objs = [objs[name] for name, _, _ in LIB_UNITS]
    if _needs(A_PATH, lib_objs):
        tmp = A_PATH.with_suffix(".a.tmp")
        if tmp.exists():
            tmp.unlink()
        _run([cc, *ARCH, "--lib", *[str(o) for o in lib_objs], "-o", str(tmp)])
        os.replace(tmp, A_PATH)
    return SO_PATH


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(SO_PATH)
