"""Restart files in the reference's layout: write / read round trips (the
written files also read back with scipy's independent netCDF reader, with
the reference's variable names, dimension order and fill value), and a run
started from a restart of the reference's check/case_00 final state on the
device against the oracle (read_restart: parameters and states from the
file, no soil-moisture initialisation, Muskingum coefficients from the file)."""
from types import SimpleNamespace

import numpy as np
import pytest

from mhm_gb300 import restart
from oracle import oracle

import test_case00_run as run_case


PER_SCENE = {name for name, dims in restart.EFF_PARAMS.values() if dims[:1] == ("scene",)}


def _grid_mask():
    m = np.zeros((5, 4), bool)          # [ncols][nrows]
    m[1:, 1:] = True
    m[0, 2] = True
    return m


def test_mhm_restart_round_trip(tmp_path):
    mask = _grid_mask()
    n, H = int(mask.sum()), 3
    rng = np.random.default_rng(1)
    states = {k: rng.uniform(0, 100, n) for k in ("interc", "snowpack", "sealSTW", "unsatSTW", "satSTW")}
    states["soilMoist"] = rng.uniform(0, 100, H * n)
    scenes = []
    for s in range(2):
        p = {name: rng.uniform(0.1, 1.0, n) for name in ("fSealed", "alpha", "degDayInc", "degDayMax",
                                                          "degDayNoPre", "karstLoss", "kFastFlow", "kSlowFlow",
                                                          "kBaseFlow", "kPerco", "tempThresh", "unsatThresh",
                                                          "sealedThresh", "fAsp")}
        for name in ("fRoots", "soilMoistSat", "soilMoistFC", "wiltingPoint", "soilMoistExp"):
            p[name] = rng.uniform(0.1, 1.0, H * n)
        p["maxInter"] = rng.uniform(0.1, 1.0, 12 * n)
        scenes.append(p)
    hd = np.array([50.0, 300.0, 1000.0])
    path = tmp_path / "mhm_restart.nc"
    restart.write_mhm_restart(path, mask, states, scenes, hd)
    r = restart.read_mhm_restart(path)
    assert np.array_equal(r.mask, mask) and r.n_scenes == 2 and np.array_equal(r.horizon_depth, hd)
    for k, v in states.items():
        assert np.array_equal(r.states[k], v), k
    for s in range(2):
        got = r.eff_params(s)
        for k, v in scenes[s].items():
            # scene-independent parameters keep the last scene's values, as in the reference's file
            want = v if k in PER_SCENE else scenes[-1][k]
            assert np.array_equal(got[k], want), (s, k)
    from scipy.io import netcdf_file
    with netcdf_file(str(path), "r", mmap=False) as f:
        sm = f.variables["L1_soilMoist"]
        assert sm.dimensions == ("L1_SoilHorizons", "ncols1", "nrows1")
        assert f.variables["L1_fRoots"].dimensions == ("L1_LandCoverPeriods", "L1_SoilHorizons", "ncols1", "nrows1")
        assert f.variables["L1_maxInter"].dimensions == ("L1_LAITimesteps", "ncols1", "nrows1")
        assert sm._FillValue == restart.NODATA
        grid = np.array(sm.data)
        assert np.all(grid[:, ~mask] == restart.NODATA)
        assert np.array_equal(grid[:, mask].reshape(-1), states["soilMoist"])


def test_mhm_restart_with_a_gridded_lai_series(tmp_path):
    """18 LAI entries (a monthly series): L1_LAITimesteps has 18 entries and
    they come back as the series (n_lai, lai_params)"""
    mask = _grid_mask()
    n, H = int(mask.sum()), 2
    rng = np.random.default_rng(2)
    states = {k: rng.uniform(0, 100, n) for k in ("interc", "snowpack", "sealSTW", "unsatSTW", "satSTW")}
    states["soilMoist"] = rng.uniform(0, 100, H * n)
    p = {name: rng.uniform(0.1, 1.0, n) for name in ("fSealed", "karstLoss", "fAsp")}
    p["maxInter"] = rng.uniform(0.1, 1.0, 18 * n)
    path = tmp_path / "series_restart.nc"
    restart.write_mhm_restart(path, mask, states, [p], np.array([200.0, 1000.0]))
    r = restart.read_mhm_restart(path)
    assert r.n_lai == 18
    assert np.array_equal(r.lai_params(0)["maxInter"].reshape(-1), p["maxInter"])
    from scipy.io import netcdf_file
    with netcdf_file(str(path), "r", mmap=False) as f:
        assert f.dimensions["L1_LAITimesteps"] == 18


@pytest.mark.gpu
def test_gpu_restart_with_a_gridded_lai_series(tmp_path):
    """a run with a monthly LAI series, written as restart files and resumed
    in a new context, continues bit for bit as the first context does"""
    from mhm_gb300 import synth
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(12, 10, 2, l11_factor=2, seed=8, jul_start=2447893)
    p = synth.make_eff_params(dom, seed=9)
    n_lai = 4
    series = np.random.default_rng(10).uniform(0.1, 3.0, (n_lai, dom.n_cells))
    f = synth.make_forcing(dom, 24 * 60, seed=11)
    a = MhmGpu(dom)
    try:
        a.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
        a.set_lai_series(-2, n_lai)
        a.set_lai_params(series)
        a.set_meteo(1, **f)
        a.run(1, 24 * 20)
        pw = dict(a.get_eff_params(0))
        pw["maxInter"] = series.reshape(-1)
        a.write_restart(tmp_path / "m.nc", [pw], mrm_path=tmp_path / "r.nc")
        q_cont = a.run(24 * 20 + 1, 24 * 40)
    finally:
        a.close()
    b = MhmGpu(dom, read_states=True)
    try:
        b.set_routing_params(synth.ROUTING_PARAMS_DEFAULT)
        b.set_lai_series(-2, n_lai)
        b.load_restart(restart.read_mhm_restart(tmp_path / "m.nc"), mrm=restart.read_mrm_restart(tmp_path / "r.nc"))
        b.set_meteo(1, **f)
        q_res = b.run(24 * 20 + 1, 24 * 40)
    finally:
        b.close()
    assert np.array_equal(q_cont, q_res)


def test_mrm_restart_round_trip(tmp_path):
    z = np.load(run_case.FIX)
    mask = np.ones((6, 1), bool)
    n = 6
    rng = np.random.default_rng(2)
    st = {"qOUT": rng.uniform(0, 9, n), "Qmod": rng.uniform(0, 9, n), "qTIN": rng.uniform(0, 9, 2 * n),
          "qTR": rng.uniform(0, 9, 2 * n), "C1": np.r_[rng.uniform(0, 1, n - 1), 0.0],
          "C2": np.r_[rng.uniform(0, 1, n - 1), 0.0]}
    net = {"fromN": np.array([1, 2, 3, 4, 5, -9999], np.int32), "toN": np.array([2, 3, 4, 5, 6, -9999], np.int32),
           "netPerm": np.array([1, 2, 3, 4, 5, -9999], np.int32), "rOrder": np.array([1, 2, 3, 4, 5, -9999], np.int32),
           "length": rng.uniform(1e3, 5e3, n - 1), "slope": rng.uniform(1e-4, 1e-2, n - 1),
           "fFPimp": rng.uniform(0, 1, (2, n - 1)), "L11_L1_Id": np.arange(1, n + 1, dtype=np.int32),
           "L1_L11_Id": np.arange(1, n + 1, dtype=np.int32), "gaugeNodeList": np.array([6], np.int32)}
    path = tmp_path / "mrm_restart.nc"
    restart.write_mrm_restart(path, mask, st, net, 3600.0, mask1=mask)
    r = restart.read_mrm_restart(path)
    assert r.ts_rout == 3600.0
    for k, v in st.items():
        assert np.array_equal(r.states[k], v), k
    for k, v in net.items():
        assert np.array_equal(r.network[k], v), k
    assert z["from_n"].size == 34    # the case_00 fixture's network, which the GPU test writes


def case00_restart(tmp_path):
    """check/case_00's final state (restart goldens) with the 1991 scene's
    parameters, written to restart files and read back."""
    z, doms, forcing = run_case.load_run()
    gamma, procs, gold = run_case.case_setup("case_00")
    p, rp = run_case.regionalised("hmath", gamma)
    n = int(z["l1_area_km2"].size)
    mask = np.ones((n, 1), bool)
    st = {k: gold["s_L1_" + v] for k, v in (("interc", "Inter"), ("snowpack", "snowPack"), ("sealSTW", "sealSTW"),
                                             ("unsatSTW", "unsatSTW"), ("satSTW", "satSTW"))}
    st["soilMoist"] = gold["s_L1_soilMoist"].reshape(-1)
    rst = {"qOUT": gold["s_L11_qOUT"], "Qmod": gold["s_L11_Qmod"], "C1": gold["s_L11_C1"], "C2": gold["s_L11_C2"],
           "qTIN": np.asarray(np.load(run_case.FIX)["gold_L11_qTIN"]).reshape(-1),
           "qTR": np.asarray(np.load(run_case.FIX)["gold_L11_qTR"]).reshape(-1)}
    restart.write_mhm_restart(tmp_path / "b1_mHM_restart.nc", mask, st, [p[0], p[1]], np.array([200.0, 1000.0]))
    restart.write_mrm_restart(tmp_path / "b1_mRM_restart.nc", mask, rst,
                              {"fromN": z["from_n"], "toN": z["to_n"], "netPerm": z["net_perm"]})
    return (restart.read_mhm_restart(tmp_path / "b1_mHM_restart.nc"),
            restart.read_mrm_restart(tmp_path / "b1_mRM_restart.nc"), doms[1], forcing, rp)


@pytest.mark.gpu
def test_gpu_run_from_case00_restart(tmp_path):
    from mhm_gb300.model import MhmGpu
    mhm, mrm, dom, forcing, rp = case00_restart(tmp_path)
    days = 30
    dom = SimpleNamespace(**dict(vars(dom), jul_start=dom.jul_start + 546))     # 1991-07-01
    f = {k: np.ascontiguousarray(v[:days]) for k, v in forcing.items()}       # reused daily rows
    g = MhmGpu(dom, proc_soilmoist=1, proc_pet=0, proc_routing=1, hourly=False, read_states=True)
    try:
        g.load_restart(mhm, 1, mrm)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"], f["tmin"], f["tmax"])
        q = g.run(1, days * 24)[0, 0]
        st = g.get_state(0)
    finally:
        g.close()
    o = oracle.OracleRun(dom, mhm.eff_params(1), rout_param=rp, proc_rout=1, hourly=False, read_states=True)
    for k, v in (("interc", "interc"), ("snowpack", "snowpack"), ("sealSTW", "sealSTW"), ("unsat", "unsatSTW"),
                 ("sat", "satSTW"), ("SM", "soilMoist")):
        np.copyto(o.state[k], mhm.states[v])
    for k in ("qOUT", "Qmod", "qTIN", "qTR", "C1", "C2"):
        np.copyto(o.state[k], mrm.states[k])
    qo, _, _ = o.run(f, 1, 1, days * 24)
    assert np.array_equal(q, qo[:, 0])
    assert np.array_equal(st["soilMoist"], o.state["SM"])
    assert np.array_equal(st["satSTW"], o.state["sat"])
    assert np.array_equal(st["Qmod"], o.state["Qmod"])
    # the restart's soil moisture was used: step 1 did not reset it to 0.5 FC
    assert not np.array_equal(mhm.states["soilMoist"], 0.5 * mhm.eff_params(1)["soilMoistFC"])


@pytest.mark.parametrize("case", run_case.OUTPUT_CASES)
def test_restart_parameter_set_of_the_check_cases(case, tmp_path):
    """With the process cases given, the writer emits the effective
    parameters the reference's restart of that check case holds: no more,
    no fewer (the process-dependent ones: Jarvis threshold, LAI/aspect
    factors, Hargreaves-Samani coefficient, Priestley-Taylor alpha)."""
    gamma, (proc_sm, proc_pet, proc_rout), _ = run_case.case_setup(case)
    z = np.load(run_case.FIX if case == "case_00" else run_case.GOLD_DIR / f"{case.replace('_', '')}_gold.npz")
    ref_vars = {str(v) for v in z["gold_restart_vars" if case == "case_00" else "restart_vars"]}
    p, _ = run_case.regionalised("hmath", gamma, proc_sm, proc_pet, proc_rout)
    n, H = p[0]["fSealed"].size, run_case.H
    names = {"jarvis_c1": "jarvis_thresh_c1", "SMs": "soilMoistSat", "FC": "soilMoistFC", "PW": "wiltingPoint",
             "beta": "soilMoistExp"}
    scenes = [{names.get(k, k): v for k, v in q.items()} for q in p]
    states = {k: np.zeros(n) for k in ("interc", "snowpack", "sealSTW", "unsatSTW", "satSTW")}
    states["soilMoist"] = np.zeros(H * n)
    path = tmp_path / "r.nc"
    restart.write_mhm_restart(path, np.ones((n, 1), bool), states, scenes, np.array([200.0, 1000.0]),
                              proc_sm=proc_sm, proc_pet=proc_pet)
    from scipy.io import netcdf_file
    with netcdf_file(str(path), "r", mmap=False) as f:
        ours = set(f.variables)
    assert ours & set(restart.EFF_PARAMS) == ref_vars & set(restart.EFF_PARAMS), case
