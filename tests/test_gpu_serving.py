"""The serving loop: requests admitted into running batches as slots free up
give exactly the discharge of the same request run alone."""
import numpy as np
import pytest

from mhm_gb300 import serve

pytestmark = pytest.mark.gpu


def test_results_equal_alone_and_in_the_mix():
    basins = serve.make_catalogue(2, seed=3, n_min=150, n_max=600)
    chunk = 24
    srv = serve.Server(basins, hbm_budget=8e9, chunk=chunk, max_slots=3, spinup_steps=48)
    reqs = serve.make_requests(basins, 7, rate=200.0, seed=5, h_min_days=1, h_max_days=4)
    summary = srv.serve(reqs, timeout_s=300)
    assert summary["requests"] == 7
    assert srv.iterations > max(r.horizon for r in reqs) // chunk  # batches really overlapped in time
    for r in reqs:
        alone = serve.run_alone(basins[r.basin], r, chunk)
        mixed = r.discharge()
        assert mixed.shape == alone.shape
        assert np.array_equal(mixed, alone), r.rid
        assert r.latency >= 0


def test_admission_respects_the_budget():
    basins = serve.make_catalogue(2, seed=3, n_min=150, n_max=600)
    one = max(serve.context_bytes(b, 2, 24) for b in basins)
    srv = serve.Server(basins, hbm_budget=one * 1.2, chunk=24, max_slots=2, spinup_steps=24)
    reqs = serve.make_requests(basins, 4, rate=1000.0, seed=8, h_min_days=1, h_max_days=2)
    srv.serve(reqs, timeout_s=300)
    assert len(srv.finished) == 4
    assert srv.used == 0
