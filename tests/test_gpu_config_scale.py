"""Parity at the sizes of the measured workloads, through the C ABI.

* The plain basin (L1 96 x 96 cells, 3 horizons, L0 = L1/4, effective
  parameters from mpr() of the parameter namelist's default values, one year
  of 8,760 hourly steps, tilted-plane DEM): gauge discharge of every step and
  every restart state at the end of the year, bit for bit against the
  oracle's hmath build and within 1e-9 relative against its libm build (the
  C library's exp/log/pow, i.e. the reference's arithmetic).  The whole year
  is where threshold branches (mo_soil_moisture.f90:233, mo_runoff.f90:139)
  would let last-bit differences compound (the time loop of
  src/mHM/mo_mhm_eval.f90:136-150).
* The calibration ensemble (L1 200 x 200, 3 horizons, 256 parameter sets
  within the namelist bounds, 720 hourly steps) run as ONE 256-member context
  in both register variants the autotuner chooses between: the outlet
  discharge of 16 members spread over the member dimension equals, bit for
  bit, 16 independent oracle runs (oracle MPR of that set + oracle time loop).
* The single large domain (L1 1000 x 1000 = 1e6 cells, 6 horizons, 62,500 L11
  nodes in 1478 levels, spatially correlated precipitation, L0 = L1/2,
  default parameters) for one 240-step chunk -- the instantiation the bench
  times (PET input with the Feddes stress, lean variant) in all three
  register variants, and with the routing wavefront walked by one 16-CTA
  cluster launch: gauge discharge, total runoff and every restart state bit
  for bit against the hmath oracle.
"""
import numpy as np
import pytest

from mhm_gb300 import params, synth

pytestmark = pytest.mark.gpu

STATE_MAP = {"interc": "interc", "snowpack": "snowpack", "sealSTW": "sealSTW", "unsatSTW": "unsat",
             "satSTW": "sat", "soilMoist": "SM", "qOUT": "qOUT", "Qmod": "Qmod", "qTIN": "qTIN", "qTR": "qTR",
             "C1": "C1", "C2": "C2"}
REL_TOL_LIBM = 1e-9   # the reference-parity bound for FP64 discharge and states


def bitwise(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(a - b)
    return float(np.max(np.where(d == 0.0, 0.0, d / np.maximum(np.abs(b), 1e-300))))


def _eff(ref: dict) -> dict:
    return {k: v for k, v in ref.items() if k not in ("Wd", "slope_emp", "horizon_depth")}


def test_plain_basin_full_year_against_both_oracles():
    from mhm_gb300.model import MhmGpu
    from oracle import oracle
    dom = synth.make_domain(96, 96, 3, 4, seed=1, dem_kind="plane")
    l0 = synth.make_l0(dom, 4, seed=4)
    gam = params.default_gamma(1, 0, 1, l0.n_geo)
    off = params.offsets(1, 0, 1, l0.n_geo)
    rp = gam[off[7]:off[7] + 5]
    T, B = 8760, 720
    g = MhmGpu(dom)
    try:
        g.mpr_setup(l0)
        g.mpr(gam)
        g.init_states(0)
        p_dev = g.get_eff_params(0)
        p_h = _eff(oracle.oracle_mpr(dom.n_cells, 3, l0, gam, off, 1, 0, "hmath"))
        p_l = _eff(oracle.oracle_mpr(dom.n_cells, 3, l0, gam, off, 1, 0, "libm"))
        for k, v in p_h.items():
            assert bitwise(p_dev[k], v), k
        o_h = oracle.OracleRun(dom, p_h, rout_param=rp, kind="hmath")
        o_l = oracle.OracleRun(dom, p_l, rout_param=rp, kind="libm")
        q_d, q_h, q_l = [], [], []
        for tt0 in range(1, T + 1, B):
            n = min(B, T + 1 - tt0)
            f = synth.make_forcing(dom, n, seed=2, t0=tt0)
            g.set_meteo(tt0, **f)
            q_d.append(g.run(tt0, n)[0].T)
            q_h.append(o_h.run(f, tt0, tt0, n)[0])
            q_l.append(o_l.run(f, tt0, tt0, n)[0])
        st = g.get_state()
    finally:
        g.close()
    q_d, q_h, q_l = (np.concatenate(x) for x in (q_d, q_h, q_l))
    assert q_d.shape == (T, 1) and np.all(np.isfinite(q_d)) and q_d.max() > 0
    assert bitwise(q_d, q_h), f"gauge Q vs hmath oracle: max rel {max_rel(q_d, q_h)}"
    assert max_rel(q_d, q_l) <= REL_TOL_LIBM, max_rel(q_d, q_l)
    for k, ko in STATE_MAP.items():
        assert bitwise(st[k], o_h.state[ko]), f"state {k}: max rel {max_rel(st[k], o_h.state[ko])}"
        assert max_rel(st[k], o_l.state[ko]) <= REL_TOL_LIBM, (k, max_rel(st[k], o_l.state[ko]))


@pytest.fixture(scope="module")
def ensemble():
    from oracle import oracle
    dom = synth.make_domain(200, 200, 3, 4, seed=1, dem_kind="fractal", fractal_beta=3.0, tilt=0.001)
    l0 = synth.make_l0(dom, 4, seed=4)
    gam = params.random_gammas(256, 1, 0, 1, l0.n_geo, seed=3)
    off = params.offsets(1, 0, 1, l0.n_geo)
    T = 720
    f = synth.make_forcing(dom, T, seed=2)
    checked = list(range(0, 256, 16))
    q_ref = {}
    for m in checked:
        p = _eff(oracle.oracle_mpr(dom.n_cells, 3, l0, gam[m], off, 1, 0, "hmath"))
        run = oracle.OracleRun(dom, p, rout_param=gam[m][off[7]:off[7] + 5], kind="hmath")
        q_ref[m] = run.run(f, 1, 1, T)[0][:, 0]
    return dom, l0, gam, f, T, q_ref


@pytest.mark.parametrize("occ", ["4", "8"])
def test_ensemble_256_members_equal_independent_oracle_runs(ensemble, occ, monkeypatch):
    from mhm_gb300.model import MhmGpu
    dom, l0, gam, f, T, q_ref = ensemble
    monkeypatch.setenv("MHM_CELL_OCC", occ)
    g = MhmGpu(dom, n_members=256)
    try:
        g.mpr_setup(l0)
        g.mpr(gam)
        for m in range(256):
            g.init_states(m)
        g.set_meteo(1, **f)
        q = g.run(1, T)          # [M][gauges][T]
    finally:
        g.close()
    assert np.all(np.isfinite(q))
    for m, qr in q_ref.items():
        assert bitwise(q[m, 0], qr), (m, max_rel(q[m, 0], qr))
    # members differ from each other (their parameter sets do)
    assert not np.array_equal(q[0, 0], q[16, 0])


@pytest.fixture(scope="module")
def large():
    from oracle import oracle
    dom = synth.make_domain(1000, 1000, 6, 4, seed=1, dem_kind="fractal", fractal_beta=3.0, tilt=0.0005, ridges=6)
    l0 = synth.make_l0(dom, 2, seed=4)
    gam = params.default_gamma(1, 0, 1, l0.n_geo)
    off = params.offsets(1, 0, 1, l0.n_geo)
    f = synth.make_forcing_grf(dom, 240, seed=2)
    return dom, l0, gam, off, f, oracle


@pytest.mark.parametrize("occ,cluster", [("4", "0"), ("6", "0"), ("8", "0"), ("8", "16")])
def test_large_domain_one_chunk_bitwise(large, occ, cluster, monkeypatch):
    from mhm_gb300.model import MhmGpu
    dom, l0, gam, off, f, oracle = large
    assert dom.n_cells == 1_000_000 and dom.n_nodes == 62_500 and dom.depth_stats()[0] == 1478
    monkeypatch.setenv("MHM_CELL_OCC", occ)
    monkeypatch.setenv("MHM_ROUTE_CLUSTER", cluster)   # 16: the routing wavefront in one cluster launch
    g = MhmGpu(dom)
    try:
        g.mpr_setup(l0)
        g.mpr(gam)
        g.init_states(0)
        g.enable_outputs(total_runoff=True)
        g.set_meteo(1, **f)
        q = g.run(1, 240)[0].T
        tro, _ = g.get_outputs()
        st = g.get_state()
        p = g.get_eff_params(0)
    finally:
        g.close()
    key = f"o_{occ}_c{cluster}"
    if not hasattr(test_large_domain_one_chunk_bitwise, "ref"):
        # the oracle time loop from the device's effective parameters (the
        # regionalisation itself is pinned bit for bit by tests/test_mpr.py)
        run = oracle.OracleRun(dom, p, rout_param=gam[off[7]:off[7] + 5], kind="hmath")
        qo, troo, _ = run.run(f, 1, 1, 240, want_tro=True)
        test_large_domain_one_chunk_bitwise.ref = (qo, troo, run.state)
    qo, troo, sto = test_large_domain_one_chunk_bitwise.ref
    assert bitwise(q, qo), (key, max_rel(q, qo))
    assert bitwise(tro[:, 0], troo), (key, max_rel(tro[:, 0], troo))
    for k, ko in STATE_MAP.items():
        assert bitwise(st[k], sto[ko]), (key, k, max_rel(st[k], sto[ko]))
