"""Routing case 3 (each link's celerity from its L0 river path): the host
celerity against the oracle's restatement of L11_calc_celerity bit for bit,
and the device's routing with those celerities against the oracle (routing
step, C1/C2, discharge and states), for a routing step both shorter and
longer than the model step."""
import ctypes as C

import numpy as np
import pytest

from mhm_gb300 import routing, synth
from oracle import oracle

SLOPE_FACTOR = 30.0   # &routing3 slope_factor (mhm_parameter.nml value)


def _paths(n_links, seed, slope_scale):
    rng = np.random.default_rng(seed)
    n = rng.integers(1, 9, n_links)
    ptr = np.concatenate([[0], np.cumsum(n)])
    return ptr, rng.uniform(0.1, slope_scale, int(ptr[-1]))


def test_link_celerity_matches_oracle():
    ptr, sl = _paths(200, 1, 40.0)
    got = routing.link_celerity(SLOPE_FACTOR, ptr, sl)
    L = oracle.load("hmath")
    dp = C.POINTER(C.c_double)
    want = [L.ora_link_celerity(SLOPE_FACTOR, np.ascontiguousarray(sl[ptr[i]:ptr[i + 1]]).ctypes.data_as(dp),
                                int(ptr[i + 1] - ptr[i])) for i in range(200)]
    assert np.array_equal(got, np.array(want))
    with pytest.raises(ValueError):
        routing.link_celerity(SLOPE_FACTOR, [0, 0], [])


@pytest.mark.gpu
@pytest.mark.parametrize("cellsize,l11_factor,slope_scale", [(250.0, 2, 40.0), (3000.0, 4, 0.2)])
def test_gpu_routing_case3_bitwise(cellsize, l11_factor, slope_scale):
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(12, 10, 3, l11_factor=l11_factor, seed=1, cellsize_m=cellsize)
    ptr, sl = _paths(dom.n_links, 7, slope_scale)
    cel = routing.link_celerity(SLOPE_FACTOR, ptr, sl)
    L = oracle.load("hmath")
    dp = C.POINTER(C.c_double)
    c1, c2 = np.zeros(dom.n_links), np.zeros(dom.n_links)
    ts = L.ora_update_param_links(cel.ctypes.data_as(dp), 0.0, np.ascontiguousarray(dom.length).ctypes.data_as(dp),
                                  dom.n_links, c1.ctypes.data_as(dp), c2.ctypes.data_as(dp))
    assert ts != 3600.0            # one of the adaptive modes: several passes per step, or windows
    p = synth.make_eff_params(dom, seed=3)
    T = 96
    f = synth.make_forcing(dom, T, seed=2, gamma_theta=4.0)
    g = MhmGpu(dom, proc_routing=3)
    try:
        g.prepare(p)
        g.set_link_celerity(cel)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        q = np.concatenate([g.run(1, 48), g.run(49, 48)], axis=2)[0, 0]
        st = g.get_state(0)
    finally:
        g.close()
    o = oracle.OracleRun(dom, p, rout_param=[0.0], proc_rout=3, link_celerity=cel)
    qo, _, _ = o.run(f, 1, 1, 48)
    qo2, _, _ = o.run(f, 1, 49, 48)
    assert np.array_equal(q, np.concatenate([qo[:, 0], qo2[:, 0]]))
    assert np.array_equal(st["C1"][: dom.n_links], c1) and np.array_equal(st["C2"][: dom.n_links], c2)
    for k, ok in (("soilMoist", "SM"), ("qTR", "qTR"), ("qTIN", "qTIN"), ("Qmod", "Qmod"), ("qOUT", "qOUT")):
        assert np.array_equal(np.asarray(st[k]).reshape(-1), o.state[ok].reshape(-1)[: np.asarray(st[k]).size]), k
