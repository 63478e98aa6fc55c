"""Generates tests/golden/reference_weno.npz by running the reference's own WENO advection kernel
(kernel2DXYWENOADVp, compiled unchanged from the reference sources by oracle/ref_build.py) on the GPU.

Run on a GPU machine that has oracle/_ref/custen_ref_sm103a.cubin:
    python tests/golden/make_golden_weno.py [output.npz]
Inputs are regenerated from their seeds (weno_inputs below); only the configurations and the reference
outputs are stored. tests/test_weno_oracle.py checks the CPU oracle against these fixtures.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from custen_gb300.buffers import DeviceBuffer  # noqa: E402
from custen_gb300.inputs import weno_inputs  # noqa: E402

# (nx, ny, numTiles, BLOCK_X, BLOCK_Y, rough): at least two blocks per direction and per tile, as the
# reference kernel assumes
CONFIGS = [
    (64, 48, 1, 16, 8, 0),
    (96, 64, 2, 32, 8, 1),
    (64, 96, 3, 16, 16, 0),
    (128, 128, 4, 32, 8, 1),
    (48, 32, 1, 8, 8, 1),
]


def run(cfg, seed):
    nx, ny, tiles, bx, by, rough = cfg
    f, u, v, dx, dy = weno_inputs(nx, ny, seed, rough=bool(rough))
    bufs = [DeviceBuffer.from_array(a) for a in (f, u, v)]
    out = DeviceBuffer.from_array(np.zeros_like(f))
    oracle.reference_weno(nx, ny, tiles, bx, by, out.ptr, bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, 1.0 / dx, 1.0 / dy)
    return out.download((ny, nx), np.float64)


def main(path: str) -> None:
    if oracle.reference_kernels() is None:
        raise SystemExit("reference cubin not present")
    arrays = {"configs": np.array(CONFIGS, dtype=np.int64)}
    for i, cfg in enumerate(CONFIGS):
        arrays[f"out_{i}"] = run(cfg, 200 + i)
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {len(CONFIGS)} configurations")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).with_name("reference_weno.npz")))
