"""Multiscale parameter regionalisation: start-up parity (host), oracle
consistency (CPU) and the device MPR against the oracle (GPU).

The device MPR evaluates the reference's per-L0-cell expressions once per
(soil type, land cover) pair and sums in the reference's block order, so its
L1 parameters must equal the oracle's (hmath build) bit for bit."""
import ctypes as C

import numpy as np
import pytest

from mhm_gb300 import params, synth
from oracle import oracle

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)

PROC_CASES = [(1, 0), (2, 1), (3, -1), (4, 0)]


def _dom_l0(H=3, nr=12, nc=10, factor=4, holes=0.1, seed=4, lat_shift=0.0):
    dom = synth.make_domain(nr, nc, H, l11_factor=2, seed=1)
    l0 = synth.make_l0(dom, factor, seed=seed, holes=holes, lat_shift=lat_shift)
    return dom, l0


def test_gamma_layout_matches_namelist_rows():
    for sm in (1, 2, 3, 4):
        for pet in (-1, 0, 1):
            for rout in (0, 1):
                off = params.layout(sm, pet, rout, 4)
                rows = params.rows(sm, pet, rout, 4)
                assert off[10] == len(rows)
                names = [r[0] for r in rows]
                assert names[off[0]] == "canopyInterceptionFactor"
                assert names[off[1]] == "snowTreshholdTemperature"
                assert names[off[2]] == "orgMatterContent_forest"
                assert names[off[3]] == "imperviousStorageCapacity"
                assert names[off[5]] == "interflowStorageCapacityFactor"
                assert names[off[6]] == "rechargeCoefficient"
                assert names[off[8]] == "GeoParam(1,:)"
                if rout == 1:
                    assert names[off[7]] == "muskingumTravelTime_constant"


def test_soil_weights_and_slope_emp_match_oracle(lib, ora_hmath):
    dom, l0 = _dom_l0(H=6, nr=20, nc=16)
    H = dom.n_horizons
    nS, mH = l0.n_soil, l0.max_hor
    hd_a = l0.horizon_depth.copy()
    wd_a = np.zeros(nS * H * mH)
    rc = lib.mhm_soil_weights(nS, mH, l0.soil_n_hor.ctypes.data_as(_ip), l0.soil_ud.ctypes.data_as(_dp),
                              l0.soil_ld.ctypes.data_as(_dp), l0.soil_rz_depth.ctypes.data_as(_dp), H,
                              hd_a.ctypes.data_as(_dp), wd_a.ctypes.data_as(_dp))
    assert rc == 0
    hd_b = l0.horizon_depth.copy()
    wd_b = np.zeros_like(wd_a)
    rc = ora_hmath.ora_soil_weights(nS, mH, l0.soil_n_hor.ctypes.data_as(_ip), l0.soil_ud.ctypes.data_as(_dp),
                                    l0.soil_ld.ctypes.data_as(_dp), l0.soil_rz_depth.ctypes.data_as(_dp), H,
                                    hd_b.ctypes.data_as(_dp), wd_b.ctypes.data_as(_dp))
    assert rc == 0
    assert np.array_equal(wd_a, wd_b) and np.array_equal(hd_a, hd_b)
    assert hd_a[-1] == l0.soil_rz_depth[-1]  # the last soil type's depth is left behind
    w = wd_a.reshape(nS, H, mH)
    pos = np.where(w > 0, w, 0).sum(-1)
    assert np.all(np.abs(pos - 1.0) < 1e-6)
    # slope_emp: ranks / (n + 1), ties (0.1 degree grid) share the later rank
    se_a = np.zeros(l0.n_cells0)
    se_b = np.zeros(l0.n_cells0)
    assert lib.mhm_slope_emp(l0.n_cells0, l0.slope0.ctypes.data_as(_dp), se_a.ctypes.data_as(_dp)) == 0
    ora_hmath.ora_slope_emp(l0.n_cells0, l0.slope0.ctypes.data_as(_dp), se_b.ctypes.data_as(_dp))
    assert np.array_equal(se_a, se_b)
    s = l0.slope0
    for v in np.unique(s)[:20]:
        assert np.unique(se_a[s == v]).size == 1
    order = np.argsort(s, kind="stable")
    assert np.all(np.diff(se_a[order]) >= 0)


def test_soil_weights_reject_shallow_soil(lib):
    nh = np.array([2], np.int32)
    ud = np.array([0.0, 300.0])
    ld = np.array([300.0, 400.0])
    rz = np.array([400.0])
    hd = np.array([200.0, 500.0, 900.0])   # 500 reaches below the 400 mm soil
    wd = np.zeros(3 * 2)
    rc = lib.mhm_soil_weights(1, 2, nh.ctypes.data_as(_ip), ud.ctypes.data_as(_dp), ld.ctypes.data_as(_dp),
                              rz.ctypes.data_as(_dp), 3, hd.ctypes.data_as(_dp), wd.ctypes.data_as(_dp))
    assert rc != 0


@pytest.mark.parametrize("proc_sm,proc_pet", PROC_CASES)
def test_oracle_mpr_constraints(proc_sm, proc_pet):
    dom, l0 = _dom_l0(H=4, lat_shift=-55.0 if proc_pet == 0 else 0.0)
    off = params.layout(proc_sm, proc_pet, 1, l0.n_geo)
    for seed in (0, 1):
        g = params.random_gammas(1, proc_sm, proc_pet, 1, l0.n_geo, seed=seed)[0]
        r = oracle.oracle_mpr(dom.n_cells, 4, l0, g, off, proc_sm, proc_pet, "hmath")
        N, H = dom.n_cells, 4
        fr = r["fRoots"].reshape(H, N)
        assert np.allclose(fr.sum(0), 1.0, rtol=0, atol=1e-12)
        sms, fc, pw = (r[k].reshape(H, N) for k in ("soilMoistSat", "soilMoistFC", "wiltingPoint"))
        assert np.all(pw <= fc) and np.all(fc <= sms) and np.all(pw > 0)
        assert np.all(r["kFastFlow"] >= 1.0) and np.all(r["kFastFlow"] <= r["kSlowFlow"])
        assert np.all(r["kSlowFlow"] >= 2.0) and np.all(r["kBaseFlow"] >= r["kSlowFlow"])
        assert np.all(r["kPerco"] >= 2.0)
        assert np.allclose(r["fSealed"], 0.6 * (r["fSealed"] / 0.6))
        # libm restatement within 1e-9 of the hmath one
        q = oracle.oracle_mpr(N, 4, l0, g, off, proc_sm, proc_pet, "libm")
        for k in ("soilMoistSat", "soilMoistFC", "wiltingPoint", "fRoots", "kSlowFlow", "alpha", "kPerco",
                  "unsatThresh", "petLAIcorFactor"):
            a, b = r[k], q[k]
            assert np.allclose(a, b, rtol=1e-9, atol=0), k


# ---------------------------------------------------------------- GPU ----
def _gpu_vs_oracle(proc_sm, proc_pet, H=3, nr=12, nc=10, factor=4, holes=0.1, n_members=3, gridded=False,
                   lat_shift=0.0):
    from mhm_gb300.model import MhmGpu
    dom, l0 = _dom_l0(H=H, nr=nr, nc=nc, factor=factor, holes=holes, lat_shift=lat_shift)
    if gridded:
        l0.gridded_lai = True
    off = params.layout(proc_sm, proc_pet, 1, l0.n_geo)
    gam = params.random_gammas(n_members, proc_sm, proc_pet, 1, l0.n_geo, seed=11)
    g = MhmGpu(dom, proc_soilmoist=proc_sm, proc_pet=proc_pet, n_members=n_members)
    try:
        g.mpr_setup(l0)
        g.mpr(gam)
        ref0 = oracle.oracle_mpr(dom.n_cells, H, l0, gam[0], off, proc_sm, proc_pet, "hmath")
        for name in ("Wd", "slope_emp", "horizon_depth"):
            assert np.array_equal(g.mpr_aux(name), ref0[name]), name
        for m in range(n_members):
            ref = ref0 if m == 0 else oracle.oracle_mpr(dom.n_cells, H, l0, gam[m], off, proc_sm, proc_pet,
                                                         "hmath")
            got = g.get_eff_params(m)
            for name, arr in got.items():
                want = ref[name]
                if name == "fAsp" and proc_pet == -1:
                    continue  # not computed by the reference in that case
                assert np.array_equal(arr, want), (m, name, np.max(np.abs(arr - want)))
    finally:
        g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("proc_sm,proc_pet", PROC_CASES)
def test_gpu_mpr_bitwise(proc_sm, proc_pet):
    _gpu_vs_oracle(proc_sm, proc_pet, lat_shift=-55.0 if proc_sm == 4 else 0.0)


@pytest.mark.gpu
def test_gpu_mpr_gridded_lai_and_six_horizons():
    _gpu_vs_oracle(3, -1, H=6, gridded=True, holes=0.0, nr=16, nc=9, factor=3)


@pytest.mark.gpu
def test_gpu_mpr_then_run_matches_oracle_chain():
    """MPR -> cell chain -> routing on the GPU equals oracle MPR -> oracle run."""
    from mhm_gb300.model import MhmGpu
    dom, l0 = _dom_l0(H=3)
    off = params.layout(1, 0, 1, l0.n_geo)
    gam = params.random_gammas(2, 1, 0, 1, l0.n_geo, seed=5)
    T = 72
    forc = synth.make_forcing(dom, T, seed=2)
    g = MhmGpu(dom, proc_soilmoist=1, proc_pet=0, n_members=2)
    try:
        g.mpr_setup(l0)
        g.mpr(gam)
        for m in range(2):
            g.init_states(m)
        g.set_meteo(1, forc["pre"], forc["temp"], forc["pet"])
        q = g.run(1, T)
    finally:
        g.close()
    for m in range(2):
        ref = oracle.oracle_mpr(dom.n_cells, 3, l0, gam[m], off, 1, 0, "hmath")
        p = {k: v for k, v in ref.items() if k not in ("Wd", "slope_emp", "horizon_depth")}
        run = oracle.OracleRun(dom, p, rout_param=gam[m][off[7]:off[7] + 5], proc_sm=1, proc_pet=0)
        qo, _, _ = run.run(forc, 1, 1, T)
        assert np.array_equal(q[m, 0], qo[:, 0]), m
