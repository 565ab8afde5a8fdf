"""The reference's regression case check/case_04: domains with their own
start dates, warm-up lengths and resolutions, pinned end to end.

  domain 1: L1 = L11 = 24 km, 1990-01-02 .. 1990-12-31, 180 warm-up days
  domain 2: L1 = 12 km under a 24 km routing grid -- the many-to-one L1 -> L11
            accumulation of L11_runoff_acc (src/mRM/mo_mrm_pre_routing.f90:
            77-143) with 109 L1 cells on 34 nodes -- 1990-07-05 .. 1992-12-31
            across the land-cover scene switch of 1991-01-01
  domain 4: 24 km, 1989-07-06 .. 1990-12-31, 360 warm-up days
  domain 5: L1 = L11 = 12 km (109 nodes), 1991-11-12 .. 1992-12-31

Every run takes the effective parameters of the domain's own restart file
(the regionalisation is pinned by the other cases) and the network mRM
built; forcing is the test_domain's 24 km daily meteo on the L1 cells.
Checked on the oracle (libm and hmath builds) and on the device: the daily
discharge equals b<d>_daily_discharge.out to its 7 decimals and the file
byte for byte; final states bit-identical for the libm build, within 1e-12
for the hmath build and the device, which equals the hmath build bit for
bit.  Fixture: tests/golden/case04_gold.npz (tests/golden/make_case04_domains.py)."""
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from mhm_gb300 import outputs, params
from oracle import oracle

import test_case00_mpr as mpr_case
from test_case00_run import HMATH_RTOL, Q_DECIMALS, check_states, daily_means, load_run

GOLD = Path(__file__).resolve().parent / "golden" / "case04_gold.npz"
DOMAINS = [1, 2, 4, 5]
KEYS = {"fSealed": "fSealed", "alpha": "alpha", "degDayInc": "degDayInc", "degDayMax": "degDayMax",
        "degDayNoPre": "degDayNoPre", "fAsp": "fAsp", "karstLoss": "karstLoss", "kfastFlow": "kFastFlow",
        "kSlowFlow": "kSlowFlow", "kBaseFlow": "kBaseFlow", "kPerco": "kPerco", "tempThresh": "tempThresh",
        "unsatThresh": "unsatThresh", "sealedThresh": "sealedThresh", "maxInter": "maxInter", "fRoots": "fRoots",
        "soilMoistSat": "soilMoistSat", "soilMoistFC": "soilMoistFC", "wiltingPoint": "wiltingPoint",
        "soilMoistExp": "soilMoistExp"}


def case04(d: int):
    """(domain per land-cover scene, parameters per scene, routing parameters,
    forcing, run description, golds) of domain d."""
    z0 = load_run()[0]                    # case_00's meteo tables and soil horizons (case_04 uses the same)
    z = np.load(GOLD)
    pre = f"d{d}_"
    g = lambda k: z[pre + k]                                       # noqa: E731
    n1, n11 = int(g("l1_area_km2").size), int(g("l11_area_km2").size)
    doms, ps = [], []
    for scene in range(2):
        doms.append(SimpleNamespace(
            n_cells=n1, n_horizons=2, n_nodes=n11, n_outlets=1, timestep=1, jul_start=int(g("jul_start")),
            evap_coeff=z0["evap_coeff"], fday_prec=1.0 - z0["fnight_prec"], fnight_prec=z0["fnight_prec"],
            fday_pet=1.0 - z0["fnight_pet"], fnight_pet=z0["fnight_pet"], fday_temp=-1.0 * z0["fnight_temp"],
            fnight_temp=z0["fnight_temp"], l1_area_km2=g("l1_area_km2"), l1_l11_id=g("l1_l11_id"),
            l11_area_km2=g("l11_area_km2"), l11_l1_id=g("l11_l1_id"), net_perm=g("net_perm"),
            from_n=g("from_n"), to_n=g("to_n"), length=g("length"), slope=g("slope"),
            ffp_imp=np.ascontiguousarray(g("ffp_imp")[scene]), gauge_node=g("gauge_node"),
            latitude=g("latitude"), horizon_depth=np.array([200.0, 1000.0])))
        p = {}
        for rname, key in KEYS.items():
            a = g("p_" + rname)
            if a.ndim >= 2 and rname != "maxInter":            # [scene][...]: scene-dependent parameter
                a = a[scene]
            p[key] = np.ascontiguousarray(a, np.float64).reshape(-1)
        ps.append(p)
    gamma = mpr_case.load_case()[2]
    off = params.layout(1, 0, 1, 10)
    rp = gamma[off[7]:off[8]]
    forcing = {k: g(k) for k in ("pre", "temp", "pet")}
    run = dict(n_steps=int(g("sim_days")) * 24, warm_days=int(g("warming_days")), scene0=int(g("scene0")),
               s2=int(g("scene2_from_day")) * 24 if int(g("scene2_from_day")) > 0 else -1)
    gold = {"q": g("q_sim"), "q_obs": g("q_obs"), "ids": g("gauge_ids"), "text": bytes(g("text"))}
    gold.update({k[len(pre):]: z[k] for k in z.files if k.startswith(pre + "s_")})
    return doms, ps, rp, forcing, run, gold


def segments(run):
    """(scene, first step, steps) of the run's land-cover periods"""
    if run["s2"] > 0:
        return [(0, 1, run["s2"]), (1, run["s2"] + 1, run["n_steps"] - run["s2"])]
    return [(run["scene0"], 1, run["n_steps"])]


def check_discharge(d, gold, q_steps, run):
    qd = daily_means(q_steps, run["warm_days"])
    assert np.array_equal(np.round(qd, Q_DECIMALS), gold["q"][:, 0]), (d, np.abs(qd - gold["q"][:, 0]).max())
    jul_eval = int(np.load(GOLD)[f"d{d}_jul_start"]) + run["warm_days"]
    text = outputs.format_daily_discharge(jul_eval, list(gold["ids"]), gold["q_obs"], qd[:, None])
    assert text.encode() == gold["text"], d


def oracle_run(doms, ps, rp, forcing, run, kind):
    kw = dict(rout_param=rp, proc_sm=1, proc_pet=0, proc_rout=1, hourly=False, kind=kind)
    qs, prev = [], None
    for scene, t0, n in segments(run):
        r = oracle.OracleRun(doms[scene], ps[scene], **kw)
        if prev is not None:               # states carry over into the new land-cover scene
            for k, v in prev.state.items():
                if k not in ("C1", "C2"):
                    np.copyto(r.state[k], v)
        qs.append(r.run(forcing, 1, t0, n)[0][:, 0])
        prev = r
    st = dict(prev.state)
    st["soilMoist"] = st.pop("SM")
    st["unsatSTW"], st["satSTW"] = st.pop("unsat"), st.pop("sat")
    return np.concatenate(qs), st


@pytest.mark.parametrize("kind", ["libm", "hmath"])
@pytest.mark.parametrize("domain", DOMAINS)
def test_oracle_reproduces_case04(domain, kind):
    doms, ps, rp, forcing, run, gold = case04(domain)
    q, st = oracle_run(doms, ps, rp, forcing, run, kind)
    check_discharge(domain, gold, q, run)
    bad = check_states(gold, st, 0.0 if kind == "libm" else HMATH_RTOL)
    assert not bad, (domain, kind, bad)


@pytest.mark.gpu
@pytest.mark.parametrize("domain", DOMAINS)
def test_gpu_reproduces_case04(domain):
    from mhm_gb300.model import MhmGpu
    doms, ps, rp, forcing, run, gold = case04(domain)
    segs = segments(run)
    g = MhmGpu(doms[segs[0][0]], proc_soilmoist=1, proc_pet=0, proc_routing=1, hourly=False, n_members=1)
    try:
        qs = []
        for i, (scene, t0, n) in enumerate(segs):
            g.set_eff_params(ps[scene])
            if i == 0:
                g.init_states(0)
                g.set_meteo(1, forcing["pre"], forcing["temp"], forcing["pet"])
            else:                          # land-cover scene switch: new parameters, states kept
                g.set_link_fpimp(doms[scene].ffp_imp)
            g.set_routing_params(rp)
            qs.append(g.run(t0, n)[0, 0])
        st = g.get_state(0)
    finally:
        g.close()
    q = np.concatenate(qs)
    check_discharge(domain, gold, q, run)
    bad = check_states(gold, st, HMATH_RTOL)
    assert not bad, (domain, bad)
    oq, _ = oracle_run(doms, ps, rp, forcing, run, "hmath")
    assert np.array_equal(oq, q)
