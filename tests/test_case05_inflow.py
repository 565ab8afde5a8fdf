"""Inflow gauges pinned by the reference's own regression case check/case_05.

case_05 runs three domains on case_00's test_domain inputs (same parameters,
processes, period and network), each evaluated at gauges 398 (the outlet)
and 333, where gauge 333 is also an inflow gauge: not a headwater in domain 1
(its daily discharge replaces the node's runoff and the links draining into
the node are cut, src/mRM/mo_mrm_pre_routing.f90:179-214 and
src/mRM/mo_mrm_routing.f90:447-452), a headwater in domain 2 (added to the
node's runoff), absent in domain 3.  case_05 reads a monthly gridded LAI
series (timeStep_LAI_input = -2, src/common/mo_common_datetime_type.f90:
138-155) whose file is not in the reference tree, so the time loop here runs
with the effective parameters of the reference's own restart files (the
regionalisation is pinned by the other cases), the 18 monthly maxInter
entries of the run (1990-01 .. 1991-06) as the context's gridded LAI series.

Checked for every domain, on the oracle (libm and hmath builds) and on the
device: the 365 daily discharges of both gauges equal b<d>_daily_discharge.out
rounded to its 7 decimals and the file itself byte for byte; every final
state of b<d>_mHM/mRM_restart_00<d>.nc is bit-identical for the libm build
and within 1e-12 for the hmath build and the device, which equals the hmath
build bit for bit.  Fixture: tests/golden/case05_gold.npz
(tests/golden/make_case05_inflow.py)."""
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from mhm_gb300 import outputs, params
from oracle import oracle

import test_case00_mpr as mpr_case
from test_case00_run import HMATH_RTOL, Q_DECIMALS, check_states, daily_means, load_run

GOLD = Path(__file__).resolve().parent / "golden" / "case05_gold.npz"
N_LAI = 18       # monthly LAI entries of the run, 1990-01 .. 1991-06
H = 2
KEYS = {"fSealed": "fSealed", "alpha": "alpha", "degDayInc": "degDayInc", "degDayMax": "degDayMax",
        "degDayNoPre": "degDayNoPre", "fAsp": "fAsp", "karstLoss": "karstLoss", "kfastFlow": "kFastFlow",
        "kSlowFlow": "kSlowFlow", "kBaseFlow": "kBaseFlow", "kPerco": "kPerco", "tempThresh": "tempThresh",
        "unsatThresh": "unsatThresh", "sealedThresh": "sealedThresh", "fRoots": "fRoots",
        "soilMoistSat": "soilMoistSat", "soilMoistFC": "soilMoistFC", "wiltingPoint": "wiltingPoint",
        "soilMoistExp": "soilMoistExp"}


def case05(d: int):
    """(domains per land-cover scene, effective parameters per scene, routing
    parameters, inflow gauges, golds) of domain d."""
    z0, doms, forcing = load_run()
    z = np.load(GOLD)
    pre = f"d{d}_"
    n = doms[0].n_cells
    doms = [SimpleNamespace(**dict(vars(dm), gauge_node=z[pre + "gauge_node"])) for dm in doms]
    ps = []
    for scene in range(2):
        p = {}
        for rname, key in KEYS.items():
            a = z[pre + "p_" + rname]
            if a.ndim >= 2:                        # [scene][...]: scene-dependent parameter
                a = a[scene]
            p[key] = np.ascontiguousarray(a, np.float64).reshape(-1)
        p["maxInter"] = np.ascontiguousarray(z[pre + "p_maxInter"]).reshape(-1)  # [18 LAI months][cell]
        ps.append(p)
    gamma = mpr_case.load_case()[2]
    off = params.layout(1, 0, 1, 10)
    rp = gamma[off[7]:off[8]]
    inflow = None
    if z[pre + "inflow_node"].size:
        inflow = dict(node=z[pre + "inflow_node"], headwater=z[pre + "inflow_headwater"], day0=1,
                      q=np.ascontiguousarray(z["inflow_q333"][:, None]))
    gold = {"q": z[pre + "q_sim"], "q_obs": z[pre + "q_obs"], "ids": z[pre + "gauge_ids"],
            "text": bytes(z[pre + "text"])}
    gold.update({k[len(pre):]: z[k] for k in z.files if k.startswith(pre + "s_")})
    return z0, doms, forcing, ps, rp, inflow, gold


def monthly(p):
    """the parameters with 12 monthly maxInter slots (the first 12 series entries;
    the series replaces them in the run)"""
    q = dict(p)
    q["maxInter"] = p["maxInter"][: 12 * (p["maxInter"].size // N_LAI)]
    return q


def check_discharge(z0, gold, q_steps, warm_days):
    qd = np.stack([daily_means(q_steps[:, i], warm_days) for i in range(q_steps.shape[1])], axis=1)
    assert np.array_equal(np.round(qd, Q_DECIMALS), gold["q"]), np.abs(qd - gold["q"]).max()
    text = outputs.format_daily_discharge(int(z0["jul_start"]) + warm_days, list(gold["ids"]), gold["q_obs"], qd)
    assert text.encode() == gold["text"]


def oracle_run(doms, ps, rp, inflow, forcing, s2, n_steps, kind):
    kw = dict(rout_param=rp, proc_sm=1, proc_pet=0, proc_rout=1, hourly=False, kind=kind, inflow=inflow,
              lai_mode=-2, n_lai=N_LAI)
    r1 = oracle.OracleRun(doms[0], ps[0], **kw)
    q1, _, _ = r1.run(forcing, 1, 1, s2)
    r2 = oracle.OracleRun(doms[1], ps[1], **kw)
    for k, v in r1.state.items():          # states carry over into the new land-cover scene
        if k not in ("C1", "C2"):
            np.copyto(r2.state[k], v)
    q2, _, _ = r2.run(forcing, 1, s2 + 1, n_steps - s2)
    st = dict(r2.state)
    st["soilMoist"] = st.pop("SM")
    st["unsatSTW"], st["satSTW"] = st.pop("unsat"), st.pop("sat")
    return q1, np.concatenate([q1, q2]), st


@pytest.mark.parametrize("kind", ["libm", "hmath"])
@pytest.mark.parametrize("domain", [1, 2, 3])
def test_oracle_reproduces_case05(domain, kind):
    z0, doms, forcing, ps, rp, inflow, gold = case05(domain)
    n_steps, warm = int(z0["sim_days"]) * 24, int(z0["warming_days"])
    s2 = int(z0["scene2_from_day"]) * 24
    _, q, st = oracle_run(doms, ps, rp, inflow, forcing, s2, n_steps, kind)
    check_discharge(z0, gold, q, warm)
    bad = check_states(gold, st, 0.0 if kind == "libm" else HMATH_RTOL)
    assert not bad, (domain, kind, bad)


@pytest.mark.gpu
@pytest.mark.parametrize("domain", [1, 2, 3])
def test_gpu_reproduces_case05(domain):
    from mhm_gb300.model import MhmGpu
    z0, doms, forcing, ps, rp, inflow, gold = case05(domain)
    n_steps, warm = int(z0["sim_days"]) * 24, int(z0["warming_days"])
    s2 = int(z0["scene2_from_day"]) * 24
    g = MhmGpu(doms[0], proc_soilmoist=1, proc_pet=0, proc_routing=1, hourly=False, n_members=1)
    try:
        g.set_eff_params(monthly(ps[0]))
        g.set_routing_params(rp)
        g.init_states(0)
        g.set_lai_series(-2, N_LAI)
        g.set_lai_params(ps[0]["maxInter"].reshape(N_LAI, -1))
        if inflow is not None:
            g.set_inflow_gauges(inflow["node"], inflow["headwater"], inflow["q"], day0=1)
        g.set_meteo(1, forcing["pre"], forcing["temp"], forcing["pet"])
        q1 = g.run(1, s2)[0].T
        g.set_eff_params(monthly(ps[1]))   # land-cover scene 1991: new parameters, states kept
        g.set_link_fpimp(doms[1].ffp_imp)
        g.set_routing_params(rp)
        q2 = g.run(s2 + 1, n_steps - s2)[0].T
        st = g.get_state(0)
    finally:
        g.close()
    q = np.concatenate([q1, q2])
    check_discharge(z0, gold, q, warm)
    bad = check_states(gold, st, HMATH_RTOL)
    assert not bad, (domain, bad)
    o1, oq, _ = oracle_run(doms, ps, rp, inflow, forcing, s2, n_steps, "hmath")
    assert np.array_equal(oq, q)
