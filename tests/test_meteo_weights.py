"""read_meteo_weights: daily forcing spread over the day by hourly weights
L1_{pre,pet,temp}_weights(cell, month, hour) (temporal_disagg_meteo_weights,
src/meteo/mo_meteo_temporal_tools.f90:32-50, used by
src/meteo/mo_meteo_handler.f90:1102-1107, 1183-1189, 1265-1270), on the
check/case_00 basin with daily forcing.

The oracle's weights path, given the weights that restate the day/night
ratios, reproduces the day/night run (a weight read at the wrong hour or
month would move day/night boundaries and miss by orders of magnitude);
the device equals the oracle bit for bit with random weights."""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import oracle

import test_case00_run as run_case

DAYS = 120


def weights_like_daynight(dom):
    """[24][12][N] weights equal to the day/night ratios of `dom` (isday: 6 < hour <= 18)."""
    N = dom.n_cells
    hours = np.arange(24)
    isday = (hours > 6) & (hours <= 18)
    out = {}
    for name, ratio in (("pre", "prec"), ("pet", "pet")):
        fd, fn = getattr(dom, "fday_" + ratio), getattr(dom, "fnight_" + ratio)
        w = np.where(isday[:, None], 2.0 * fd[None, :] / 24.0, 2.0 * fn[None, :] / 24.0)
        out[name] = np.ascontiguousarray(np.repeat(w[:, :, None], N, axis=2))
    out["temp"] = np.ones((24, 12, N))
    return out


def random_weights(n, seed=3):
    rng = np.random.default_rng(seed)
    return {"pre": rng.uniform(0.0, 0.2, (24, 12, n)), "pet": rng.uniform(0.0, 0.2, (24, 12, n)),
            "temp": 1.0 + 0.01 * rng.standard_normal((24, 12, n))}


def _setup():
    z, doms, forcing = run_case.load_run()
    gamma, procs, gold = run_case.case_setup("case_00")
    dom = SimpleNamespace(**dict(vars(doms[0]), fday_temp=np.zeros(12), fnight_temp=np.zeros(12)))
    p, rp = run_case.regionalised("hmath", gamma)
    return dom, forcing, p[0], rp, gamma


def _oracle_run(dom, forcing, p, rp, weights=None):
    r = oracle.OracleRun(dom, p, rout_param=rp, proc_sm=1, proc_pet=0, proc_rout=1, hourly=False, kind="hmath",
                         meteo_weights=weights)
    q, _, _ = r.run(forcing, 1, 1, DAYS * 24)
    return q[:, 0], r.state


def test_oracle_weights_restating_the_daynight_ratios():
    dom, forcing, p, rp, _ = _setup()
    q_dn, st_dn = _oracle_run(dom, forcing, p, rp)
    q_w, st_w = _oracle_run(dom, forcing, p, rp, weights_like_daynight(dom))
    assert np.allclose(q_w, q_dn, rtol=1e-9, atol=1e-12)
    for k in ("interc", "snowpack", "sealSTW", "SM", "unsat", "sat", "qOUT"):
        assert np.allclose(st_w[k], st_dn[k], rtol=1e-9, atol=1e-12), k
    # random weights change the run
    q_r, _ = _oracle_run(dom, forcing, p, rp, random_weights(dom.n_cells))
    assert not np.allclose(q_r, q_dn, rtol=1e-3)


@pytest.mark.gpu
def test_gpu_meteo_weights_bitwise():
    from mhm_gb300.model import MhmGpu
    import test_case00_mpr as mpr_case
    dom, forcing, p, rp, gamma = _setup()
    w = random_weights(dom.n_cells)
    l0_for = mpr_case.load_case()[0]
    g = MhmGpu(dom, proc_soilmoist=1, proc_pet=0, proc_routing=1, hourly=False, n_members=1)
    try:
        g.mpr_setup(l0_for(1))
        g.mpr(gamma)
        last = g.get_eff_params(0)
        g.mpr_setup(l0_for(0))
        g.mpr(gamma)
        p0 = g.get_eff_params(0)
        for k in run_case.SCENE_INDEPENDENT:
            p0[k] = last[k]
        g.set_eff_params(p0)
        g.init_states(0)
        g.set_meteo_weights(w["pre"], w["pet"], w["temp"])
        g.set_meteo(1, forcing["pre"], forcing["temp"], forcing["pet"])
        q = g.run(1, DAYS * 24)[0, 0]
        st = g.get_state(0)
        g.set_meteo_weights()            # back to the day/night ratios
        g.init_states(0)
        q_dn = g.run(1, DAYS * 24)[0, 0]
    finally:
        g.close()
    q_o, st_o = _oracle_run(dom, forcing, p, rp, w)
    assert np.array_equal(q, q_o)
    for ours, theirs in (("interc", "interc"), ("snowpack", "snowpack"), ("sealSTW", "sealSTW"),
                         ("unsatSTW", "unsat"), ("satSTW", "sat"), ("soilMoist", "SM"), ("qOUT", "qOUT")):
        got = np.asarray(st[ours]).reshape(-1)[: st_o[theirs].size]
        assert np.array_equal(got, st_o[theirs]), ours
    q_o_dn, _ = _oracle_run(dom, forcing, p, rp)
    assert np.array_equal(q_dn, q_o_dn)
