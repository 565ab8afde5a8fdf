"""The bounds-checked build (-DMHM_BOUNDS_CHECK, libmhm_gpu_bc.so): run in a
child process on the scenarios of tests/bc_scenarios.py (member-tiled
ensemble with device MPR, chunked calls and the cluster routing walk; inflow
gauges with adaptive routing windows; members at their own steps in a fused
launch; a gridded LAI series regionalised on the device), it reports no
failed index test and gives results bit-identical to
the default build; its self-test (one failing test with no access behind it)
comes back as site 99, index 7 and is cleared once read."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


def test_bounds_checked_build(tmp_path):
    from mhm_gb300 import build
    build.build(bounds_check=True)
    out = tmp_path / "bc.npz"
    env = dict(os.environ, MHM_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, str(HERE / "bc_scenarios.py"), str(out)], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    z = np.load(out)
    assert int(z["bounds_checked"]) == 1
    assert bool(z["status_clean"])
    assert z["selftest"].tolist() == [99, 7]
    assert bool(z["after_selftest"])
    # the default build (this process) gives the same bits
    sys.path.insert(0, str(HERE))
    import bc_scenarios
    from mhm_gb300 import _lib
    assert _lib.load().mhm_bounds_checked() == 0
    res, status = bc_scenarios.run_all()
    assert all(s is None for s in status)
    for k, v in res.items():
        assert np.array_equal(np.asarray(v).view(np.uint64), z[k].view(np.uint64)), k
