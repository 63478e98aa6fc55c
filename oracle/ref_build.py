"""Builds the reference's own code from the reference sources into oracle/_ref -- TEST INFRASTRUCTURE ONLY.

Nothing is copied out of the reference: the wrappers below #include the reference files where they
lie (the reference root: $CUSTEN_REFERENCE_ROOT, else a checkout named `reference` beside this
repository, else nothing is built), and only build outputs land in
oracle/_ref (git-ignored). Where the sources are absent (e.g. on the GPU machine) nothing is built
and the prebuilt outputs are used if they are present.

Outputs:
  custen_ref_sm103a.cubin -- the thirteen cuSten kernels, unchanged, for sm_103a (oracle/ref_kernels.cu),
                             driven by oracle/ref_runner.cpp.
  custen_ref_ch_sm103a.cubin -- the device code of cuPentSpeedUp/cuPentCahnADITiming (its element-wise
                             kernels, nonLinRHS, the batched pentadiagonal solves and the two cuSten XY
                             kernels it uses), driven by oracle/ref_ch_runner.cpp. CUDA 13 removed one cudaMemPrefetchAsync
                             overload the reference calls; oracle/ref_compat.h restores it.
  libserialch.so          -- cuPentSpeedUp/serialCahnADITiming/serialCahnADI.c compiled with gcc as the
                             reference's compile.sh does (-O3, no contraction flags), its main renamed,
                             with an empty hdf5.h (the header is included but unused), wrapped by
                             oracle/ref_serial_ch.c so that its static solver functions can be called.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REF = Path(os.environ["CUSTEN_REFERENCE_ROOT"]) if os.environ.get("CUSTEN_REFERENCE_ROOT") else ROOT.parent / "reference"
OUT = HERE / "_ref"
CUBIN = OUT / "custen_ref_sm103a.cubin"
CH_CUBIN = OUT / "custen_ref_ch_sm103a.cubin"
SERIAL_SO = OUT / "libserialch.so"


def available() -> bool:
    return (REF / "cuSten" / "src" / "kernels" / "2d_x_p_kernel.cu").exists()


def _nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build_cubin() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    tmp = CUBIN.with_suffix(".cubin.tmp")
    cmd = [_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++14",
           "-include", str(HERE / "ref_compat.h"), "-I", str(ROOT), f"-DREF_ROOT={REF}", "-o", str(tmp),
           str(HERE / "ref_kernels.cu")]
    subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    os.replace(tmp, CUBIN)
    return CUBIN


def build_ch_cubin() -> Path:
    """The device code of the reference's Cahn-Hilliard GPU timing program (oracle/ref_ch_kernels.cu)."""
    OUT.mkdir(parents=True, exist_ok=True)
    stub = OUT / "hdf5_stub"
    stub.mkdir(exist_ok=True)
    (stub / "hdf5.h").write_text("/* empty: the reference program includes hdf5.h; its device code uses nothing from it */\n")
    tmp = CH_CUBIN.with_suffix(".cubin.tmp")
    cmd = [_nvcc(), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++14",
           "-include", str(HERE / "ref_compat.h"), "-I", str(ROOT), "-I", str(stub), f"-DREF_ROOT={REF}",
           "-o", str(tmp), str(HERE / "ref_ch_kernels.cu")]
    subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    os.replace(tmp, CH_CUBIN)
    return CH_CUBIN


def build_serial_ch() -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    stub = OUT / "hdf5_stub"
    stub.mkdir(exist_ok=True)
    (stub / "hdf5.h").write_text("/* empty: serialCahnADI.c includes hdf5.h but calls nothing from it */\n")
    tmp = SERIAL_SO.with_suffix(".so.tmp")
    src = REF / "cuPentSpeedUp" / "serialCahnADITiming" / "serialCahnADI.c"
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-w", "-I", str(stub), f"-DSERIAL_CH_SOURCE=\"{src}\"",
           "-Dmain=serial_ch_main", "-o", str(tmp), str(HERE / "ref_serial_ch.c"), "-lm"]
    subprocess.run(cmd, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    os.replace(tmp, SERIAL_SO)
    return SERIAL_SO


def build_if_available() -> None:
    if not available():
        return
    build_cubin()
    build_ch_cubin()
    if (HERE / "ref_serial_ch.c").exists():
        build_serial_ch()


if __name__ == "__main__":
    import sys
    if len(sys.argv) > 1:   # python oracle/ref_build.py <reference root>
        REF = Path(sys.argv[1])
    build_if_available()
    print(sorted(p.name for p in OUT.glob("*")) if OUT.exists() else "reference sources not present")
