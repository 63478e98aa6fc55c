"""Child process of tests/test_checked_build.py: representative parity cases on the checked build of
the library (CUSTEN_CHECKED=1: every kernel index check raises device error bit 1 instead of faulting).

Runs every stencil variant in FP64 (each stencil configuration, plus FP32, unaligned rows, host
memory, the reference's example functions, fused and indirect c^3 - c functions), WENO, and a CH batch
in every kernel configuration; each result is checked against the oracle. Prints the number of cases
and the device error flags; exits 1 on any mismatch or flag.
"""
import os
import sys

import numpy as np

assert os.environ.get("CUSTEN_CHECKED") == "1", "run with CUSTEN_CHECKED=1"

import custen_gb300 as cs  # noqa: E402
import oracle  # noqa: E402
from custen_gb300.buffers import DeviceBuffer  # noqa: E402
from custen_gb300.inputs import weno_inputs
from tests.test_stencil_parity import FUN_IDS, check, geometry, run_both  # noqa: E402


def main() -> int:
    assert cs.LIB_PATH.name == "libcusten_gb300_checked.so"
    cs._check(cs.lib().custen_set_device(0))
    cs.device_error(clear=True)
    cases = 0
    funs = (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN)
    for variant in range(12):
        d = 0 if variant < 4 else (1 if variant < 8 else 2)
        fun = variant in funs
        for kind in ("sym", "asym", "small"):
            geom = geometry(variant, kind)
            fun_id = -1
            if fun:
                fun_id = FUN_IDS[d][1]
                geom = {0: (5, 2, 2, 1, 0, 0), 1: (1, 0, 0, 5, 2, 2), 2: (3, 1, 1, 3, 1, 1)}[d]
            for cfg in range(cs.NUM_CONFIGS):
                nx, ny = (96, 64) if d != 1 else (48, 128)
                got, ref, st, pre = run_both(variant, nx, ny, 2, 32 if d != 1 else 16, 8, geom, fun_id=fun_id,
                                             seed=variant + cfg, config=cfg)
                check(got, ref, st, pre)
                cases += 1
        got, ref, st, pre = run_both(variant, 128, 64, 2, 32, 8, geometry(variant, "sym"), dtype=np.float32,
                                     fun_id=FUN_IDS[d][1] if fun else -1, seed=variant)
        check(got, ref, st, pre)
        got, ref, st, pre = run_both(variant, 64, 256, 4, 16, 8, geometry(variant, "asym") if not fun else
                                     {0: (5, 2, 2, 1, 0, 0), 1: (1, 0, 0, 5, 2, 2), 2: (5, 2, 2, 5, 2, 2)}[d],
                                     fun_id=FUN_IDS[d][1] if fun else -1, seed=31 + variant, mem="pinned",
                                     offload=cs.HOST)
        check(got, ref, st, pre)
        cases += 2
        if not fun:
            got, ref, st, pre = run_both(variant, 98, 56, 2, 14, 4, geometry(variant, "small"), seed=11)
            check(got, ref, st, pre)
            cases += 1
        else:
            geom = {0: (3, 1, 1, 1, 0, 0), 1: (1, 0, 0, 9, 4, 4), 2: (3, 1, 1, 3, 1, 1)}[d]
            nx, ny = (64, 64) if d != 1 else (32, 128)
            got, ref, st, pre = run_both(variant, nx, ny, 2, 16 if d != 1 else 8, 8, geom, fun_id=FUN_IDS[d][0],
                                         seed=3)
            check(got, ref, st, pre)
            cs.set_fun_fusion(False)
            got, ref, st, pre = run_both(variant, 128, 64, 2, 32, 8, {0: (5, 2, 2, 1, 0, 0), 1: (1, 0, 0, 5, 2, 2),
                                         2: (3, 1, 1, 3, 1, 1)}[d], fun_id=FUN_IDS[d][1], seed=17)
            cs.set_fun_fusion(True)
            check(got, ref, st, pre)
            cases += 2
    # WENO
    f, u, v, dx, dy = weno_inputs(160, 96, 5, rough=True)
    bufs = [DeviceBuffer.from_array(a) for a in (f, u, v)]
    out = DeviceBuffer.from_array(np.zeros_like(f))
    we = cs.WenoAdvection(160, 96, out.ptr, bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, dx=dx, dy=dy, num_tiles=2)
    we.compute()
    cs._check(cs.lib().custen_device_synchronize())
    we.destroy()
    wref = oracle.weno(f, u, v, 1 / dx, 1 / dy)
    wgot = out.download((96, 160), np.float64)
    assert np.linalg.norm(wgot - wref) / np.linalg.norm(wref) <= 1e-7
    cases += 1
    # CH batch, every kernel configuration
    sizes = [64, 160, 96]
    c0 = [np.random.default_rng(60 + k).uniform(-0.1, 0.1, (n, n)) for k, n in enumerate(sizes)]
    for cfg in range(22):
        b = cs.CahnHilliardBatch(sizes)
        b.set_config(cfg)
        for k, c in enumerate(c0):
            b.set_state(k, c)
        b.step(3)
        b.synchronize()
        for k, c in enumerate(c0):
            o = oracle.CHOracle(c)
            o.step(3)
            ocur, _ = o.fields()
            cur, _ = b.state(k)
            assert np.linalg.norm(cur - ocur) / np.linalg.norm(ocur) <= 1e-10, (cfg, k)
        b.close()
        cases += 1
    flags = cs.device_error(clear=True)
    print(f"cases {cases} flags {flags}")
    return 0 if flags == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
