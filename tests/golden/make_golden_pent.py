"""Generates tests/golden/reference_pent.npz by running the reference's own pentFactorBatch and
pentSolveBatch (compiled unchanged from the reference sources into the reference CH cubin,
oracle/ref_build.py) on the GPU.

Run on a GPU machine that has oracle/_ref/custen_ref_ch_sm103a.cubin:
    python tests/golden/make_golden_pent.py [output.npz]
Inputs are regenerated from their seeds (custen_gb300/inputs.py: pent_system); the factors and solutions the
reference kernels produce are stored. tests/test_pent_oracle.py checks the CPU oracle against them.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from custen_gb300.buffers import DeviceBuffer  # noqa: E402
from custen_gb300.inputs import pent_system  # noqa: E402

CONFIGS = [(4, 33), (5, 64), (32, 96), (61, 50)]   # (m, batch)


def main(path: str) -> None:
    if not oracle.ReferenceCahnHilliardGPU.available():
        raise SystemExit("reference CH cubin not present")
    arrays = {"configs": np.array(CONFIGS, dtype=np.int64)}
    for k, (m, batch) in enumerate(CONFIGS):
        sysm = pent_system(m, batch, k)
        bufs = [DeviceBuffer.from_array(a) for a in sysm]
        oracle.reference_pent(True, [b.ptr for b in bufs[:5]], m, batch)
        oracle.reference_pent(False, [b.ptr for b in bufs], m, batch)
        for name, buf in zip(("ds", "dl", "d", "du", "dw", "x"), bufs):
            arrays[f"{name}_{k}"] = buf.download((m, batch), np.float64)
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {len(CONFIGS)} configurations")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).with_name("reference_pent.npz")))
