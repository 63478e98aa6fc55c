"""Generates tests/golden/reference_kernels.npz by running the reference's own cuSten kernels
(compiled unchanged from the reference sources, oracle/ref_build.py) on the GPU.

Run on a GPU machine that has oracle/_ref/custen_ref_sm103a.cubin:
    python tests/golden/make_golden.py [output.npz]
Inputs are regenerated from their seeds (custen_gb300/inputs.py: field; tests/helpers.py: weights_for); only the reference
outputs, the configurations and the pre-fill are stored. tests/test_golden.py checks the CPU oracle
against these fixtures.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import custen_gb300 as cs  # noqa: E402
import oracle  # noqa: E402
from custen_gb300.buffers import DeviceBuffer  # noqa: E402
from custen_gb300.inputs import field, sentinel  # noqa: E402
from tests.helpers import weights_for  # noqa: E402

# (variant, nx, ny, tiles, bx, by, H, L, R, V, T, B, fun_id)
CONFIGS = []
for v in range(12):
    d = 0 if v < 4 else (1 if v < 8 else 2)
    fun = v in (2, 3, 6, 7, 10, 11)
    if d == 0:
        geoms = [(5, 2, 2, 1, 0, 0), (4, 2, 1, 1, 0, 0) if not fun else (3, 1, 1, 1, 0, 0)]
        funs = [1, 0]
        nx, ny, bx, by = 64, 16, 16, 4
    elif d == 1:
        geoms = [(1, 0, 0, 5, 2, 2), (1, 0, 0, 4, 1, 2) if not fun else (1, 0, 0, 9, 4, 4)]
        funs = [3, 2]
        nx, ny, bx, by = 16, 64, 8, 8
    else:
        geoms = [(5, 2, 2, 5, 2, 2), (4, 2, 1, 3, 1, 1)]
        funs = [5, 4]
        nx, ny, bx, by = 48, 32, 16, 8
    for k, g in enumerate(geoms):
        CONFIGS.append((v, nx, ny, 2 if k == 0 else 1, bx, by, *g, funs[k] if fun else -1))


def run(cfg, seed):
    v, nx, ny, tiles, bx, by, H, L, R, V, T, B, fun_id = cfg
    inp = field(nx, ny, seed)
    if fun_id >= 0:
        ncoef = {0: 1, 1: 5, 2: 9, 3: 5, 4: H * V, 5: H * V}[fun_id]
        coef = np.random.default_rng(50 + seed).uniform(-1, 1, ncoef)
    else:
        coef = weights_for(v, H, V, seed)
        ncoef = coef.size
    pre = sentinel(nx, ny)
    d_in, d_out, d_c = DeviceBuffer.from_array(inp), DeviceBuffer.from_array(pre), DeviceBuffer.from_array(coef)
    d = 0 if v < 4 else (1 if v < 8 else 2)
    num_sten = H * V if d == 2 else (H if d == 0 else V)
    oracle.reference_compute(v, nx, ny, tiles, bx, by, d_out.ptr, d_in.ptr, d_c.ptr, num_sten=num_sten, H=H, L=L,
                             R=R, V=V, T=T, B=B, num_coe=ncoef,
                             func=oracle.reference_fun_ptr(fun_id) if fun_id >= 0 else 0)
    return d_out.download((ny, nx), np.float64)


def main(out_path):
    cs.build()
    if oracle.reference_kernels() is None:
        raise SystemExit("reference cubin missing")
    data = {"configs": np.array(CONFIGS, dtype=np.int32)}
    for i, cfg in enumerate(CONFIGS):
        data[f"out_{i}"] = run(cfg, seed=100 + i)
    np.savez_compressed(out_path, **data)
    print(f"wrote {len(CONFIGS)} reference outputs to {out_path}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).with_name("reference_kernels.npz")))
