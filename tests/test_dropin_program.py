"""A C++ program written against cuSten.h, linked against this library's libcuSten.a with nvcc
-rdc=true (the reference's own build model), runs on the GPU and gives the oracle's results: the
drop-in path, including a Fun device function defined in the user's translation unit (GPU)."""
import math
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import custen_gb300 as cs
import oracle

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "dropin" / "dropin_program.cu"


@pytest.fixture(scope="module")
def program_outputs(tmp_path_factory):
    cs.build()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    d = tmp_path_factory.mktemp("dropin")
    exe = d / "dropin_program"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-rdc=true", "-std=c++17", "-O2",
           "-I", str(ROOT / "include"), str(SRC), str(ROOT / "custen_gb300" / "libcuSten.a"), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe), str(d / "run")], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and "ok" in out.stdout, out.stdout + out.stderr
    nx, ny = 256, 128

    def load(name):
        return np.fromfile(d / f"run_{name}.bin", dtype=np.float64).reshape(ny, nx)
    return load, nx, ny


def test_xyp_compute_swap_compute(program_outputs):
    load, nx, ny = program_outputs
    dx, dy = 2 * math.pi / nx, 2 * math.pi / ny
    w = np.array([1, 0, -1, 0, 0, 0, -1, 0, 1], dtype=np.float64) / (4 * dx * dy)
    a = load("input")
    b1 = np.zeros_like(a)
    oracle.stencil(cs.XYP, b1, a, w, num_tiles=2, block_x=32, block_y=8, H=3, L=1, R=1, V=3, T=1, B=1)
    assert np.array_equal(load("xyp_1"), b1)
    a2 = np.zeros_like(a)
    oracle.stencil(cs.XYP, a2, b1, w, num_tiles=2, block_x=32, block_y=8, H=3, L=1, R=1, V=3, T=1, B=1)
    assert np.array_equal(load("xyp_2"), a2)


def test_user_device_function_across_translation_units(program_outputs):
    load, nx, ny = program_outputs
    a = load("input")
    coe = np.array([(0.5 if k % 2 == 0 else -0.25) + 0.125 * k for k in range(9)])
    ref = np.full_like(a, -7.0)
    st = oracle.stencil(cs.XYNPFUN, ref, a, coe, num_tiles=2, block_x=32, block_y=8, H=3, L=1, R=1, V=3, T=1, B=1,
                        fun_id=4)   # the shipped id-4 function computes the same FMA chain
    got = load("xynpfun")
    assert np.array_equal(got[st == 1], ref[st == 1])
    assert (got[st != 1] == -7.0).all()


def test_x_nonperiodic_edges(program_outputs):
    load, nx, ny = program_outputs
    dx = 2 * math.pi / nx
    w = np.array([-1.0 / 12, 16.0 / 12, -30.0 / 12, 16.0 / 12, -1.0 / 12]) / (dx * dx)
    a = load("input")
    ref = np.full_like(a, 3.0)
    st = oracle.stencil(cs.XNP, ref, a, w, num_tiles=1, block_x=32, block_y=8, H=5, L=2, R=2, V=1, T=0, B=0)
    assert np.array_equal(load("xnp"), ref)
    assert (st[:, :2] == 0).all()


def test_weno_through_the_cpp_api(program_outputs):
    load, nx, ny = program_outputs
    a, u, v = load("input"), load("u"), load("v")
    ref = oracle.weno(a, u, v, nx / (2 * math.pi), ny / (2 * math.pi))
    got = load("weno")
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-7
