"""Kernel configurations and the autotuner: every configuration is bit-identical to the oracle on every
variant, and the tuner's choice round-trips through its JSON cache (GPU)."""
import json

import numpy as np
import pytest

import custen_gb300 as cs
from tests.test_stencil_parity import FUN_IDS, check, geometry, run_both

pytestmark = pytest.mark.gpu

VARIANTS = list(range(12))


@pytest.mark.parametrize("config", range(cs.NUM_CONFIGS))
@pytest.mark.parametrize("variant", VARIANTS, ids=cs.VARIANT_NAMES)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_every_configuration_matches_the_oracle(gpu, config, variant, dtype):
    d = 0 if variant < 4 else (1 if variant < 8 else 2)
    fun = variant in (cs.XPFUN, cs.XNPFUN, cs.YPFUN, cs.YNPFUN, cs.XYPFUN, cs.XYNPFUN)
    geom = geometry(variant, "sym" if fun else "asym")
    fun_id = FUN_IDS[d][1] if fun else -1
    # 256 x 128: tiles of every configuration divide it (TMA path); 2 tiles of 64 rows
    got, ref, st, pre = run_both(variant, 256, 128, 2, 32, 8, geom, dtype=dtype, fun_id=fun_id,
                                 seed=40 + variant + config, config=config)
    check(got, ref, st, pre)


@pytest.mark.parametrize("config", range(cs.NUM_CONFIGS))
def test_configurations_on_unaligned_geometry(gpu, config):
    """nx = 100, 3 tiles of 20 rows: no configuration tiles it, every one takes the plain-load path."""
    got, ref, st, pre = run_both(cs.XYNP, 100, 60, 3, 10, 4, geometry(cs.XYNP, "asym"), seed=3, config=config)
    check(got, ref, st, pre)


def test_autotune_caches_and_reuses(gpu, tmp_path):
    from custen_gb300.buffers import DeviceBuffer
    from custen_gb300.inputs import field
    from tests.helpers import weights_for
    cache = tmp_path / "tune.json"
    cs.set_tune_cache(str(cache))
    assert cs.tune_cache_path() == str(cache)
    n = 512
    H, L, R, V, T, B = 5, 2, 2, 5, 2, 2
    inp = DeviceBuffer.from_array(field(n, n, 1))
    out = DeviceBuffer(n * n * 8)
    w = DeviceBuffer.from_array(weights_for(cs.XYP, H, V, 2))
    try:
        cs.set_autotune(1)
        h = cs.Stencil(cs.XYP, n, n, out.ptr, inp.ptr, w.ptr, H=H, L=L, R=R, V=V, T=T, B=B)
        h.compute()
        cs._check(cs.lib().custen_device_synchronize())
        chosen = h.config()
        assert chosen.startswith("f64_tw")
        doc = json.loads(cache.read_text())
        entries = doc["entries"]
        assert len(entries) == 1
        (key, ent), = entries.items()
        assert ent["config"] == chosen and len(ent["ms"]) == cs.NUM_CONFIGS
        assert f"|v{cs.XYP}|f64|{n}x{n}|" in key
        h.destroy()
        # a fresh cache load in lookup-only mode gives the stored choice
        cs.set_autotune(0)
        cs.set_tune_cache(str(cache))
        h2 = cs.Stencil(cs.XYP, n, n, out.ptr, inp.ptr, w.ptr, H=H, L=L, R=R, V=V, T=T, B=B)
        h2.compute()
        assert h2.config() == chosen
        # explicit tuning of one handle
        assert h2.autotune().startswith("f64_tw")
        h2.destroy()
    finally:
        cs.set_autotune(0)
        cs.set_tune_cache(None)
