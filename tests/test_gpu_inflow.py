"""Inflow gauges: add_inflow (src/mRM/mo_mrm_pre_routing.f90:179-214) puts a
gauge's daily discharge into the L11 runoff of its node -- added for a
headwater gauge, in place of the node's own runoff otherwise -- and
L11_routing (src/mRM/mo_mrm_routing.f90:447-452) cuts the routed outflow of
every link that drains into a non-headwater gauge's node.  The device path
(inflow kernel after the accumulation, cut flag in the routing ticks) is
compared bit for bit with the oracle's restatement, for Muskingum routing and
for adaptive routing with routing steps shorter and longer than the model
step (where a routing step's inflow is the mean over its model steps)."""
import ctypes as C

import numpy as np
import pytest

from mhm_gb300 import synth

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def _gauge_nodes(dom):
    """(non-headwater node with the most upstream links, a second node with
    upstream links), 1-based, neither the outlet."""
    nl = dom.n_links
    up = np.bincount(dom.to_n[:nl] - 1, minlength=dom.n_nodes)
    outlet = int(dom.gauge_node[0]) - 1
    order = [v for v in np.argsort(-up, kind="stable") if v != outlet and up[v] > 0]
    return int(order[0]) + 1, int(order[1]) + 1


def test_oracle_add_inflow_in_list_order(ora_hmath):
    """Gauges act in list order: headwater gauges add, others replace."""
    q = np.array([1.0, 2.0, 3.0, 4.0])
    node = np.array([2, 2, 2, 4], np.int32)
    hw = np.array([1, 0, 1, 1], np.int32)
    qin = np.array([10.0, 5.0, 0.25, 0.5])
    ora_hmath.ora_add_inflow(4, hw.ctypes.data_as(_ip), node.ctypes.data_as(_ip), qin.ctypes.data_as(_dp),
                             q.ctypes.data_as(_dp))
    assert q.tolist() == [1.0, 5.25, 3.0, 4.5]


@pytest.mark.gpu
@pytest.mark.parametrize("cluster", ["0", "8"])   # per-tick graph, cluster walk
@pytest.mark.parametrize("proc_rout,cellsize,l11", [(1, 1000.0, 2), (2, 250.0, 2), (2, 3000.0, 4)])
def test_gpu_inflow_gauges_bitwise(proc_rout, cellsize, l11, cluster, monkeypatch):
    from mhm_gb300.model import MhmGpu
    monkeypatch.setenv("MHM_ROUTE_CLUSTER", cluster)
    from oracle import oracle
    dom = synth.make_domain(12, 10, 3, l11_factor=l11, seed=1, cellsize_m=cellsize)
    p = synth.make_eff_params(dom, seed=3)
    T = 96
    f = synth.make_forcing(dom, T, seed=2, gamma_theta=4.0)
    cut, add = _gauge_nodes(dom)
    node = np.array([cut, add], np.int32)
    hw = np.array([0, 1], np.int32)
    q = np.random.default_rng(9).uniform(0.5, 20.0, (6, 2))     # days 1..6
    rp = synth.ROUTING_PARAMS_DEFAULT if proc_rout == 1 else np.array([1.5, 0, 0, 0, 0])
    g = MhmGpu(dom, proc_routing=proc_rout)
    try:
        g.prepare(p, rp)
        g.set_inflow_gauges(node, hw, q, day0=1)
        g.enable_outputs(qmod=True)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        qg = np.concatenate([g.run(1, 48), g.run(49, 48)], axis=2)[0, 0]
        _, qm = g.get_outputs()
        st = g.get_state(0)
    finally:
        g.close()
    o = oracle.OracleRun(dom, p, rout_param=rp if proc_rout == 1 else [1.5], proc_rout=proc_rout,
                         inflow=dict(node=node, headwater=hw, day0=1, q=q))
    qo, _, _ = o.run(f, 1, 1, 48)
    qo2, _, qmo2 = o.run(f, 1, 49, 48, want_qmod=True)
    q_or = np.concatenate([qo[:, 0], qo2[:, 0]])
    assert np.array_equal(qg.view(np.uint64), q_or.view(np.uint64)), np.max(np.abs(qg - q_or))
    assert np.array_equal(qm[0], qmo2)
    for k, ok in (("qTR", "qTR"), ("qTIN", "qTIN"), ("Qmod", "Qmod"), ("qOUT", "qOUT")):
        assert np.array_equal(np.asarray(st[k]).reshape(-1), o.state[ok].reshape(-1)), k
    # links draining into the non-headwater gauge's node pass nothing on
    L = dom.n_nodes
    ups = [int(dom.from_n[i]) - 1 for i in range(dom.n_links) if dom.to_n[i] == cut]
    assert ups and all(st["qTR"][v] == 0.0 and st["qTR"][L + v] == 0.0 for v in ups)
    # the gauge's discharge reached the outlet: without inflow the series differs
    o0 = oracle.OracleRun(dom, p, rout_param=rp if proc_rout == 1 else [1.5], proc_rout=proc_rout)
    assert not np.array_equal(o0.run(f, 1, 1, 48)[0][:, 0], qo[:, 0])


@pytest.mark.gpu
def test_gpu_inflow_discharge_must_cover_the_run():
    from mhm_gb300.model import MhmError, MhmGpu
    dom = synth.make_domain(12, 10, 3, l11_factor=2, seed=1)
    p = synth.make_eff_params(dom, seed=3)
    f = synth.make_forcing(dom, 48, seed=2)
    g = MhmGpu(dom)
    try:
        g.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
        g.set_inflow_gauges([2], [1], np.ones((1, 1)), day0=1)      # day 1 only
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        g.run(1, 24)
        with pytest.raises(MhmError, match="inflow discharge"):
            g.run(25, 24)                                           # day 2 is missing
        with pytest.raises(MhmError, match="out of range"):
            g.set_inflow_gauges([dom.n_nodes + 1], [1])
    finally:
        g.close()
