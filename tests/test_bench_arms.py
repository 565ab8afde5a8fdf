"""The bench's GPU arm and its reference arm describe and build the same
workload: the routing order from the library and from the oracle's own
sweep agree, so both arms get the same basin, and the `config` object and
the forcing window (fixed seeds) are identical -- checked on the small
configuration, on the CPU."""
import importlib.util
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_arms_build_the_same_workload():
    from oracle import oracle
    b = _bench()
    dom_g, l0_g, gam_g, chunk_g = b.build_workload("small")
    dom_r, l0_r, gam_r, chunk_r = b.build_workload("small", order=lambda f, t, n, o: oracle.routing_order(f, t, n, o))
    assert chunk_g == chunk_r and np.array_equal(gam_g, gam_r)
    for k in ("net_perm", "r_order", "from_n", "to_n", "length", "slope", "l1_l11_id"):
        assert np.array_equal(getattr(dom_g, k), getattr(dom_r, k)), k
    assert np.array_equal(l0_g.soil_id0, l0_r.soil_id0)
    assert b.workload_config("small", dom_g, chunk_g) == b.workload_config("small", dom_r, chunk_r)
    fg, _ = b.host_forcing(dom_g, chunk_g, pinned=False)
    fr, _ = b.host_forcing(dom_r, chunk_r, pinned=False)
    for k in ("pre", "temp", "pet"):
        assert np.array_equal(fg[k], fr[k]), k
    assert abs((fg["pre"] > 0).mean() - 0.3) < 1e-3     # 70 % dry hours
