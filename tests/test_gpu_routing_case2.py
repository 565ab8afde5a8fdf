"""Routing case 2 (routing time step from a constant celerity) on the device
against the oracle, bit for bit: a routing step shorter than the model step
(several routing passes per step, discharge averaged) and a longer one
(runoff summed over a window of model steps, one pass per window, the value
standing for every step of the window); plus the oracle's own choice of the
routing step."""
import numpy as np
import pytest

from mhm_gb300 import synth
from oracle import oracle

CELERITY = 1.5  # &routing2 streamflow_celerity (mhm_parameter.nml value)


def _domain(cellsize, l11_factor):
    return synth.make_domain(12, 10, 3, l11_factor=l11_factor, seed=1, cellsize_m=cellsize)


@pytest.mark.parametrize("cellsize,l11_factor,ts_expect", [(250.0, 2, 300.0), (3000.0, 4, 7200.0)])
def test_oracle_routing_step_choice(cellsize, l11_factor, ts_expect):
    dom = _domain(cellsize, l11_factor)
    L = oracle.load("hmath")
    import ctypes as C
    nl = dom.n_links
    c1 = np.zeros(nl)
    c2 = np.zeros(nl)
    ln = np.ascontiguousarray(dom.length)
    dp = C.POINTER(C.c_double)
    ts = L.ora_update_param_case2(CELERITY, ln.ctypes.data_as(dp), nl, c1.ctypes.data_as(dp), c2.ctypes.data_as(dp))
    assert ts == ts_expect
    k = ln / CELERITY
    assert ts <= k.min() or ts == 60.0
    assert np.allclose(c1 + c2 * 0, ts / (k + 0.5 * ts))


@pytest.mark.gpu
@pytest.mark.parametrize("cluster", ["0", "16"])   # per-tick graph, cluster walk
@pytest.mark.parametrize("cellsize,l11_factor", [(250.0, 2), (3000.0, 4)])
def test_gpu_routing_case2_bitwise(cellsize, l11_factor, cluster, monkeypatch):
    monkeypatch.setenv("MHM_ROUTE_CLUSTER", cluster)
    from mhm_gb300.model import MhmGpu
    dom = _domain(cellsize, l11_factor)
    p = synth.make_eff_params(dom, seed=3)
    T = 96
    f = synth.make_forcing(dom, T, seed=2, gamma_theta=4.0)
    g = MhmGpu(dom, proc_routing=2)
    try:
        g.prepare(p, np.array([CELERITY, 0, 0, 0, 0]))
        g.enable_outputs(qmod=True)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        q = np.concatenate([g.run(1, 48), g.run(49, 48)], axis=2)[0, 0]
        _, qm = g.get_outputs()
        st = g.get_state(0)
    finally:
        g.close()
    o = oracle.OracleRun(dom, p, rout_param=[CELERITY], proc_rout=2)
    qo, _, qmo = o.run(f, 1, 1, 48, want_qmod=True)
    qo2, _, qmo2 = o.run(f, 1, 49, 48, want_qmod=True)
    assert np.array_equal(q, np.concatenate([qo[:, 0], qo2[:, 0]]))
    assert np.array_equal(qm[0], qmo2)
    for k, ok in (("soilMoist", "SM"), ("satSTW", "sat"), ("qTR", "qTR"), ("qTIN", "qTIN"), ("Qmod", "Qmod"),
                  ("qOUT", "qOUT")):
        assert np.array_equal(np.asarray(st[k]).reshape(-1), o.state[ok].reshape(-1)[: np.asarray(st[k]).size]), k
