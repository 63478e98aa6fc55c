"""The checked build (index checks that raise device error bit 1 instead of faulting) runs the parity
cases of every kernel family without raising a flag: no kernel index leaves the extent it must stay
in. The library is compiled with -DCUSTEN_CHECKED=1 on demand and exercised in a child process."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.gpu
def test_checked_build_raises_no_flag(gpu):
    gpu.build(checked=True)
    env = dict(os.environ, CUSTEN_CHECKED="1")
    r = subprocess.run([sys.executable, "-m", "tests.checked_run"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "flags 0" in r.stdout
