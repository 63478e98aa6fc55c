"""Test-only helpers: random weights for parity cases and the dense application of a batched
pentadiagonal system (residual checks). Fields, buffers and benchmark inputs come from the package
(custen_gb300.buffers, custen_gb300.inputs)."""
from __future__ import annotations

import numpy as np


def weights_for(variant: int, H: int, V: int, seed: int, dtype=np.float64, zeros: bool = True) -> np.ndarray:
    rng = np.random.default_rng(1000 + seed)
    w = rng.uniform(-2.0, 2.0, size=H * V)
    if zeros and H * V >= 4:
        w[rng.choice(H * V, size=max(1, H * V // 4), replace=False)] = 0.0
    return w.astype(dtype)


def pent_dense_apply(ds, dl, d, du, dw, x):
    """A x for the unfactored systems (same layout), for residual checks."""
    m = x.shape[0]
    y = d * x
    y[1:] += dl[1:] * x[:-1]
    y[2:] += ds[2:] * x[:-2]
    y[:-1] += du[:-1] * x[1:]
    y[:-2] += dw[:-2] * x[2:]
    return y
