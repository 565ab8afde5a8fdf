"""The asynchronous pipeline (mhm_run_async / mhm_sync): consecutive calls
overlap routing with the next cell chain; results equal the synchronous
run bit for bit, for device and for pinned-host forcing."""
import numpy as np
import pytest

from mhm_gb300 import synth
from mhm_gb300.model import MhmGpu

pytestmark = pytest.mark.gpu


def test_async_equals_sync(monkeypatch):
    dom = synth.make_domain(24, 32, 3, 4, seed=1)
    p = synth.make_eff_params(dom, seed=3)
    f = synth.make_forcing(dom, 24 * 12, seed=2)
    a = MhmGpu(dom)
    a.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
    a.set_meteo(1, **f)
    q_sync = a.run(1, 24 * 12)
    monkeypatch.setenv("MHM_CHUNK_BYTES", str(dom.n_cells * 8 * 2 * 30))  # 30-step chunks
    b = MhmGpu(dom)
    b.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
    b.set_meteo(1, **f)
    outs = [np.zeros((1, 1, 24)) for _ in range(12)]
    for d in range(12):
        b.run_async(1 + 24 * d, 24, outs[d])
    b.sync()
    q_async = np.concatenate(outs, axis=2)
    assert np.array_equal(q_async.view(np.uint64), q_sync.view(np.uint64))
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k].view(np.uint64), sb[k].view(np.uint64)), k
