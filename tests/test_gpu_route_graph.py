"""The routing wavefront replayed from captured CUDA graphs gives the same
discharge and routing states as launching its ticks one by one, over several
chunks and calls (different chunk lengths and sub-chunk sizes make different
graphs), for two members."""
import numpy as np
import pytest

from mhm_gb300 import synth


def _run(monkeypatch, graphs: bool):
    from mhm_gb300.model import MhmGpu
    monkeypatch.setenv("MHM_ROUTE_GRAPH", "1" if graphs else "0")
    monkeypatch.setenv("MHM_CHUNK_BYTES", str(2 * 2 * 48 * 48 * 8 * 40))   # 40-step chunks
    dom = synth.make_domain(48, 48, 3, l11_factor=2, seed=4)
    ps = [synth.make_eff_params(dom, seed=3 + m) for m in range(2)]
    f = synth.make_forcing(dom, 200, seed=2)
    g = MhmGpu(dom, n_members=2)
    try:
        g.prepare(ps, synth.ROUTING_PARAMS_DEFAULT)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        q = [g.run(1, 100), g.run(101, 37), g.run(138, 63)]
        st = [g.get_state(m) for m in range(2)]
    finally:
        g.close()
    return np.concatenate(q, axis=2), st


@pytest.mark.gpu
def test_gpu_route_graph_equals_launches(monkeypatch):
    qa, sa = _run(monkeypatch, True)
    qb, sb = _run(monkeypatch, False)
    assert np.array_equal(qa, qb)
    for a, b in zip(sa, sb):
        for k in ("qOUT", "Qmod", "qTIN", "qTR"):
            assert np.array_equal(a[k], b[k]), k
