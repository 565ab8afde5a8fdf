"""The reference's own regression case pins the whole hot path end to end.

check/case_00, case_10 and case_12 (test_domain, 24 km L1 = L11, 2 soil
horizons; soil-moisture cases 1, 3 and 4; PET input corrected by aspect
(case_00) or by LAI (case_10, 12); hourly steps
with daily forcing disaggregated by the day/night ratios, PET input with
aspect correction, Muskingum routing, land-cover scene 1981 for 1990 and
1991 from 1991-01-01): 181 warm-up days from 1990-01-01, then the
evaluation year.  Fixtures: tests/golden/case00_mpr.npz (regionalisation
inputs) and case00_run.npz (forcing, the network mRM built, the
reference's daily discharge output and final restart states; made by
tests/golden/make_case00_run.py).

Checked, for the oracle (libm and hmath builds) and the device: all 365
daily discharges printed in b1_daily_discharge.out equal ours rounded to its
7 decimals, and every final state of b1_mHM/b1_mRM_restart_001.nc (cell
storages, soil moisture, routing states, C1/C2) is bit-identical for the
libm build and within 1e-12 (a last-bit difference at most) for the hmath
build and the device, which also equals the hmath build bit for bit."""
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from mhm_gb300 import outputs, params
from oracle import oracle

import test_case00_mpr as mpr_case

FIX = Path(__file__).resolve().parent / "golden" / "case00_run.npz"
H = 2
Q_DECIMALS = 7           # the discharge file prints 7 decimals


def load_run():
    z = np.load(FIX)
    n = int(z["l1_area_km2"].size)
    doms = []
    for scene in range(2):
        doms.append(SimpleNamespace(
            n_cells=n, n_horizons=H, n_nodes=n, n_outlets=1, timestep=1, jul_start=int(z["jul_start"]),
            evap_coeff=z["evap_coeff"], fday_prec=1.0 - z["fnight_prec"], fnight_prec=z["fnight_prec"],
            fday_pet=1.0 - z["fnight_pet"], fnight_pet=z["fnight_pet"], fday_temp=-1.0 * z["fnight_temp"],
            fnight_temp=z["fnight_temp"], l1_area_km2=z["l1_area_km2"], l1_l11_id=z["l1_l11_id"],
            l11_area_km2=z["l11_area_km2"], l11_l1_id=z["l11_l1_id"], net_perm=z["net_perm"],
            from_n=z["from_n"], to_n=z["to_n"], length=z["length"], slope=z["slope"],
            ffp_imp=np.ascontiguousarray(z["ffp_imp"][scene]), gauge_node=z["gauge_node"], latitude=z["latitude"],
            horizon_depth=np.array([200.0, 1000.0])))
    forcing = {"pre": z["pre"], "temp": z["temp"], "pet": z["pet"], "tmin": z["tmin"], "tmax": z["tmax"],
               "netrad": z["netrad"], "eabs": z["eabs"], "windspeed": z["windspeed"]}
    return z, doms, forcing


def daily_means(q_steps, warming_days):
    """sum(Q(iS:iE)) / 24 over each evaluation day, summed in step order
    (src/mRM/mo_mrm_write.f90:138-149)."""
    return outputs.daily_discharge(q_steps, warming_days, 24)


def check_daily_text(z, qd):
    """b1_daily_discharge.out written from our daily discharge equals the
    reference's file byte for byte."""
    text = outputs.format_daily_discharge(int(z["jul_start"]) + int(z["warming_days"]), [int(z["gold_gauge_id"])],
                                          z["gold_q_obs"], qd)
    assert text.encode() == bytes(z["gold_daily_text"])


# mHM() reads these with land-cover index 1 whatever the scene
# (src/mHM/mo_mhm_interface_run.f90:439-451), and mpr() rewrites index 1 in
# every pass of its scene loop: a multi-scene run uses the values of the
# LAST scene throughout (maxInter and sealedThresh do not depend on the scene)
SCENE_INDEPENDENT = ("unsatThresh", "karstLoss", "sealedThresh", "jarvis_thresh_c1")


GOLD_DIR = Path(__file__).resolve().parent / "golden"
# check case -> (processCase(3), processCase(5), processCase(8)); all on the test_domain inputs
CASES = {"case_00": (1, 0, 1), "case_10": (3, -1, 1), "case_12": (4, -1, 1), "case_09": (1, 1, 2),
         "case_02": (2, 2, 0), "case_03": (1, 3, 1), "case_07": (1, 0, 1)}
# case_03 and case_07 are optimisations (DDS): they write the discharge and the mRM restart
# of their last (here also best) evaluation, but no flux/state file and no mHM restart
OUTPUT_CASES = [c for c in CASES if c not in ("case_03", "case_07")]


def period(case, z):
    """(model steps, warming days) of a case's run from 1990-01-01: case_07 runs
    1990-1991 without warming, the others case_00's 181 warming days and a year."""
    if case != "case_00":
        g = np.load(GOLD_DIR / f"{case.replace('_', '')}_gold.npz")
        if "sim_days" in g.files:
            return int(g["sim_days"]) * 24, int(g["warming_days"])
    return int(z["sim_days"]) * 24, int(z["warming_days"])


def case_setup(case):
    """(gamma, (proc_sm, proc_pet, proc_rout), golds) of a check case: golds has
    the daily discharge "q", final states "s_*", L1 parameters "p_*" and, for
    adaptive routing, the link lengths mRM used."""
    if case == "case_00":
        z = np.load(FIX)
        gold = {"q": z["gold_q_daily"]}
        gold.update({"s_" + k[5:]: z[k] for k in z.files if k.startswith("gold_L")})
        return mpr_case.load_case()[2], CASES[case], gold
    z = np.load(GOLD_DIR / f"{case.replace('_', '')}_gold.npz")
    gold = {"q": z["q_daily"]}
    gold.update({k: z[k] for k in z.files if k[:2] in ("s_", "p_") or k in ("length", "ts_rout")})
    return z["gamma"], CASES[case], gold


def case_domains(case, doms, gold):
    """The run's domains (per land-cover scene), with the case's link lengths."""
    if "length" not in gold:
        return doms
    return [SimpleNamespace(**dict(vars(d), length=np.ascontiguousarray(gold["length"]))) for d in doms]


def regionalised(kind, gamma, proc_sm=1, proc_pet=0, proc_rout=1):
    l0_for, _, _, n1 = mpr_case.load_case()
    off = params.layout(proc_sm, proc_pet, proc_rout, 10)
    out = []
    for scene in range(2):
        r = oracle.oracle_mpr(n1, H, l0_for(scene), gamma, off, proc_sm, proc_pet, kind)
        out.append({k: v for k, v in r.items() if k not in ("Wd", "slope_emp", "horizon_depth")})
    for k in SCENE_INDEPENDENT:
        out[0][k] = out[-1][k]
    return out, gamma[off[7]:off[8]]


def check_states(g, st, rtol=0.0):
    gold = {"qOUT": g["s_L11_qOUT"], "Qmod": g["s_L11_Qmod"],
            "C1": g["s_L11_C1"][:-1], "C2": g["s_L11_C2"][:-1]} if "s_L11_qOUT" in g else {}
    if "s_L1_Inter" in g:   # an optimisation run (case_03) writes no mHM restart
        gold.update(interc=g["s_L1_Inter"], snowpack=g["s_L1_snowPack"], sealSTW=g["s_L1_sealSTW"],
                    unsatSTW=g["s_L1_unsatSTW"], satSTW=g["s_L1_satSTW"],
                    soilMoist=g["s_L1_soilMoist"].reshape(-1))
    bad = {}
    for k, want in gold.items():
        got = np.asarray(st[k]).reshape(-1)[: want.size]
        err = float(np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-300)))
        if not (np.array_equal(got, want) or err <= rtol):
            bad[k] = err
    return bad


# The libm oracle calls the C library's exp/log/pow as the reference's build
# did and reproduces its states bit for bit; the hmath build (the device's
# functions, <= 1 ulp from the C library's) may differ in the last bit.
HMATH_RTOL = 1e-12


@pytest.mark.parametrize("case", ["case_10", "case_12", "case_09", "case_02"])
def test_oracle_mpr_reproduces_cases(case):
    gamma, (proc_sm, proc_pet, proc_rout), gold = case_setup(case)
    l0_for, _, _, n1 = mpr_case.load_case()
    off = params.layout(proc_sm, proc_pet, proc_rout, 10)
    names = dict(mpr_case.NAMES, petLAIcorFactor="petLAIcorFactor", jarvis_thresh_c1="jarvis_thresh_c1",
                 PrieTayAlpha="PrieTayAlpha")
    for scene in range(2):
        r = oracle.oracle_mpr(n1, H, l0_for(scene), gamma, off, proc_sm, proc_pet, "hmath")
        for gname, ename in names.items():
            if "p_" + gname not in gold:
                continue
            want = mpr_case.gold_for({gname: gold["p_" + gname]}, gname, scene)
            if gname == "petLAIcorFactor":
                want = gold["p_" + gname][scene].reshape(-1)
            if gname == "PrieTayAlpha":     # depends on the LAI classes only: the same in both scenes
                want = gold["p_" + gname].reshape(-1)
            if gname == "jarvis_thresh_c1":
                want = gold["p_" + gname][0] if scene == 1 else None
            if want is not None:
                assert np.array_equal(r[ename], want), (case, scene, gname)


@pytest.mark.parametrize("kind", ["libm", "hmath"])
@pytest.mark.parametrize("case", list(CASES))
def test_oracle_reproduces_case_discharge_and_states(case, kind):
    z, doms, forcing = load_run()
    gamma, (proc_sm, proc_pet, proc_rout), gold = case_setup(case)
    doms = case_domains(case, doms, gold)
    p, rp = regionalised(kind, gamma, proc_sm, proc_pet, proc_rout)
    n_steps, warm_days = period(case, z)
    s2 = int(z["scene2_from_day"]) * 24
    kw = dict(rout_param=rp, proc_sm=proc_sm, proc_pet=proc_pet, proc_rout=proc_rout, hourly=False, kind=kind)
    r1 = oracle.OracleRun(doms[0], p[0], **kw)
    q1, _, _ = r1.run(forcing, 1, 1, s2)
    r2 = oracle.OracleRun(doms[1], p[1], **kw)
    for k, v in r1.state.items():          # states carry over into the new land-cover scene
        if k not in ("C1", "C2"):
            np.copyto(r2.state[k], v)
    q2, _, _ = r2.run(forcing, 1, s2 + 1, n_steps - s2)
    q = np.concatenate([q1[:, 0], q2[:, 0]])
    qd = daily_means(q, warm_days)
    if proc_rout:
        assert np.array_equal(np.round(qd, Q_DECIMALS), gold["q"]), (case, kind, np.abs(qd - gold["q"]).max())
    if case == "case_00":
        check_daily_text(z, qd)
    st = dict(r2.state)
    st["soilMoist"] = st.pop("SM")
    st["unsatSTW"], st["satSTW"] = st.pop("unsat"), st.pop("sat")
    bad = check_states(gold, st, 0.0 if kind == "libm" else HMATH_RTOL)
    assert not bad, (case, bad)


def output_golds(case):
    """(settings, {plane name: [interval][cell]}, Qrouted [interval][node] or None)
    of a case's b1_mHM/mRM_Fluxes_States.nc."""
    z = np.load(FIX if case == "case_00" else GOLD_DIR / f"{case.replace('_', '')}_gold.npz")
    cfg = dict(interval=int(z["out_interval"]), flags=[int(f) for f in z["out_flags"]],
               interval_mrm=int(z["out_interval_mrm"]), qrouted=bool(z["out_qrouted"]))
    fs = {k[3:]: z[k] for k in z.files if k.startswith("fs_") and k != "fs_time_bnds"}
    return cfg, fs, (z["qrouted"] if "qrouted" in z.files else None)


@pytest.mark.parametrize("kind", ["libm", "hmath"])
@pytest.mark.parametrize("case", OUTPUT_CASES)
def test_oracle_reproduces_case_outputs(case, kind):
    """b1_mHM_Fluxes_States.nc (SWC, Q, PET, aET, recharge over the evaluation
    year) and b1_mRM_Fluxes_States.nc (Qrouted, daily means or the year's
    mean at every node)."""
    z, doms, forcing = load_run()
    gamma, (proc_sm, proc_pet, proc_rout), gold = case_setup(case)
    doms = case_domains(case, doms, gold)
    cfg, fs_gold, qr_gold = output_golds(case)
    p, rp = regionalised(kind, gamma, proc_sm, proc_pet, proc_rout)
    n_steps = int(z["sim_days"]) * 24
    s2 = int(z["scene2_from_day"]) * 24
    warm = int(z["warming_days"]) * 24
    kw = dict(rout_param=rp, proc_sm=proc_sm, proc_pet=proc_pet, proc_rout=proc_rout, hourly=False, kind=kind)
    r1 = oracle.OracleRun(doms[0], p[0], **kw)
    r1.enable_outputs(cfg["interval"], cfg["flags"], warm, n_steps, 400, cfg["interval_mrm"], cfg["qrouted"])
    # the last step of 1990 is written with the 1991 scene's weights
    r1.set_output_weights(s2, p[1]["fSealed"], np.reshape(p[1]["soilMoistSat"], (H, -1)))
    r1.run(forcing, 1, 1, s2)
    r2 = oracle.OracleRun(doms[1], p[1], **kw)
    for k, v in r1.state.items():
        if k not in ("C1", "C2"):
            np.copyto(r2.state[k], v)
    r2.out, r2.out_buf = r1.out, r1.out_buf     # the output datasets carry over
    r2.out.tt_w = 0
    r2.run(forcing, 1, s2 + 1, n_steps - s2)
    fs, fs_tt, qr, qr_tt = r2.read_outputs()
    names = outputs.plane_names(cfg["flags"], H)
    assert sorted(names) == sorted(fs_gold)
    assert fs.shape[0] == next(iter(fs_gold.values())).shape[0]
    tol = 0.0 if kind == "libm" else HMATH_RTOL
    for i, name in enumerate(names):
        want = fs_gold[name]
        err = np.max(np.abs(fs[:, i] - want) / np.maximum(np.abs(want), 1e-300))
        assert np.array_equal(fs[:, i], want) or err <= tol, (case, kind, name, err)
    if qr_gold is not None:
        assert qr.shape == qr_gold.shape
        err = np.max(np.abs(qr - qr_gold) / np.maximum(np.abs(qr_gold), 1e-300))
        assert np.array_equal(qr, qr_gold) or err <= tol, (case, kind, "Qrouted", err)
    assert fs_tt[-1] == n_steps


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
def test_gpu_reproduces_case_discharge_and_states(case):
    from mhm_gb300.model import MhmGpu
    z, doms, forcing = load_run()
    l0_for, _, _, n1 = mpr_case.load_case()
    gamma, (proc_sm, proc_pet, proc_rout), gold = case_setup(case)
    doms = case_domains(case, doms, gold)
    n_steps, warm_days = period(case, z)
    s2 = int(z["scene2_from_day"]) * 24
    g = MhmGpu(doms[0], proc_soilmoist=proc_sm, proc_pet=proc_pet, proc_routing=proc_rout, hourly=False,
               n_members=1)
    try:
        g.mpr_setup(l0_for(1))            # the last scene's scene-independent parameters
        g.mpr(gamma)
        last = g.get_eff_params(0)
        g.mpr_setup(l0_for(0))
        g.mpr(gamma)
        p0 = g.get_eff_params(0)
        if proc_pet == 2:   # the device's MPR of the Priestley-Taylor alpha equals the reference's restart
            assert np.array_equal(p0["PrieTayAlpha"], gold["p_PrieTayAlpha"].reshape(-1))
        for k in SCENE_INDEPENDENT:
            p0[k] = last[k]
        g.set_eff_params(p0)
        g.init_states(0)
        g.set_meteo(1, forcing["pre"], forcing["temp"], forcing["pet"], forcing["tmin"], forcing["tmax"],
                    netrad=forcing["netrad"], eabs=forcing["eabs"], windspeed=forcing["windspeed"])
        q1 = g.run(1, s2)[0, 0]
        g.mpr_setup(l0_for(1))            # land-cover scene 1991: new parameters, states kept
        g.set_link_fpimp(doms[1].ffp_imp)
        g.mpr(gamma)                      # (its scene-independent values are the ones already used)
        q2 = g.run(s2 + 1, n_steps - s2)[0, 0]
        st = g.get_state(0)
    finally:
        g.close()
    q = np.concatenate([q1, q2])
    qd = daily_means(q, warm_days)
    if proc_rout:
        assert np.array_equal(np.round(qd, Q_DECIMALS), gold["q"]), np.abs(qd - gold["q"]).max()
    if case == "case_00":
        check_daily_text(z, qd)
    bad = check_states(gold, st, HMATH_RTOL)
    assert not bad, bad
    # and the device equals the oracle's hmath build bit for bit
    p, rp = regionalised("hmath", gamma, proc_sm, proc_pet, proc_rout)
    r1 = oracle.OracleRun(doms[0], p[0], rout_param=rp, proc_sm=proc_sm, proc_pet=proc_pet, proc_rout=proc_rout,
                          hourly=False, kind="hmath")
    o1, _, _ = r1.run(forcing, 1, 1, s2)
    if proc_pet == 1:   # the device's extraterrestrial radiation uses CUDA's trigonometric functions
        assert np.allclose(o1[:, 0], q1, rtol=1e-12, atol=0)
    else:
        assert np.array_equal(o1[:, 0], q1)


@pytest.mark.gpu
@pytest.mark.parametrize("case", OUTPUT_CASES)
def test_gpu_reproduces_case_outputs(case):
    """The device's aggregated outputs against b1_mHM_Fluxes_States.nc and
    b1_mRM_Fluxes_States.nc."""
    from mhm_gb300.model import MhmGpu
    z, doms, forcing = load_run()
    l0_for, _, _, n1 = mpr_case.load_case()
    gamma, (proc_sm, proc_pet, proc_rout), gold = case_setup(case)
    doms = case_domains(case, doms, gold)
    cfg, fs_gold, qr_gold = output_golds(case)
    n_steps = int(z["sim_days"]) * 24
    s2 = int(z["scene2_from_day"]) * 24
    warm = int(z["warming_days"]) * 24
    g = MhmGpu(doms[0], proc_soilmoist=proc_sm, proc_pet=proc_pet, proc_routing=proc_rout, hourly=False,
               n_members=1)
    try:
        g.mpr_setup(l0_for(1))
        g.mpr(gamma)
        last = g.get_eff_params(0)
        g.mpr_setup(l0_for(0))
        g.mpr(gamma)
        p0 = g.get_eff_params(0)
        for k in SCENE_INDEPENDENT:
            p0[k] = last[k]
        g.set_eff_params(p0)
        g.init_states(0)
        g.enable_flux_state_outputs(cfg["flags"], cfg["interval"], warm, n_steps, max_slots=400)
        if cfg["qrouted"]:
            g.enable_routed_outputs(cfg["interval_mrm"], warm, n_steps, max_slots=400)
        # the last step of 1990 is written with the 1991 scene's weights
        g.set_output_weights(0, s2, last["fSealed"], np.reshape(last["soilMoistSat"], (H, -1)))
        g.set_meteo(1, forcing["pre"], forcing["temp"], forcing["pet"], forcing["tmin"], forcing["tmax"],
                    netrad=forcing["netrad"])
        g.run(1, s2)
        g.mpr_setup(l0_for(1))
        g.set_link_fpimp(doms[1].ffp_imp)
        g.mpr(gamma)
        g.run(s2 + 1, n_steps - s2)
        names, fs, fs_tt = g.read_flux_state_outputs()
        qr, _ = g.read_routed_outputs() if cfg["qrouted"] else (None, None)
    finally:
        g.close()
    assert sorted(names) == sorted(fs_gold) and fs_tt[-1] == n_steps
    for i, name in enumerate(names):
        want = fs_gold[name]
        err = np.max(np.abs(fs[:, i, 0] - want) / np.maximum(np.abs(want), 1e-300))
        assert np.array_equal(fs[:, i, 0], want) or err <= HMATH_RTOL, (case, name, err)
    if qr_gold is not None:
        err = np.max(np.abs(qr[:, 0] - qr_gold) / np.maximum(np.abs(qr_gold), 1e-300))
        assert qr.shape[0] == qr_gold.shape[0] and (np.array_equal(qr[:, 0], qr_gold) or err <= HMATH_RTOL), err
