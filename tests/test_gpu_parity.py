"""GPU vs oracle parity through the C ABI (mhm_run etc.).

The GPU kernels and the oracle's hmath build evaluate the same IEEE
operations in the same order with the same elementary functions, so gauge
discharge, total runoff, L11 discharge and every restart state must be
BIT-IDENTICAL.  Against the oracle's libm build (the C library's exp/log/pow,
i.e. what gfortran calls) the tolerance is the 1e-9 relative error of the
reference-parity target.  The Hargreaves/day-night variant uses CUDA's
trigonometric functions for the extraterrestrial radiation, so it is compared
at 1e-12 relative.
"""
import numpy as np
import pytest

from mhm_gb300 import synth
from mhm_gb300.model import MhmGpu
from oracle.oracle import OracleRun

pytestmark = pytest.mark.gpu

STATE_MAP = {"interc": "interc", "snowpack": "snowpack", "sealSTW": "sealSTW", "unsatSTW": "unsat",
             "satSTW": "sat", "soilMoist": "SM", "qOUT": "qOUT", "Qmod": "Qmod", "qTIN": "qTIN", "qTR": "qTR",
             "C1": "C1", "C2": "C2"}


def bitwise(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def run_pair(dom, params, forcing, n_steps, kind="hmath", proc_sm=1, proc_pet=0, hourly=True, chunks=1):
    g = MhmGpu(dom, proc_soilmoist=proc_sm, proc_pet=proc_pet, hourly=hourly)
    g.prepare(params, synth.ROUTING_PARAMS_DEFAULT)
    g.enable_outputs(total_runoff=True, qmod=True)
    g.set_meteo(1, **forcing)
    qs, tros, qms = [], [], []
    step = n_steps // chunks
    for c in range(chunks):
        n = step if c < chunks - 1 else n_steps - step * (chunks - 1)
        qs.append(g.run(1 + c * step, n))
        tro, qm = g.get_outputs()
        tros.append(tro[:, 0])
        qms.append(qm[0])
    q_gpu = np.concatenate(qs, axis=2)[0].T  # [step, gauge]
    st_gpu = g.get_state()
    o = OracleRun(dom, params, synth.ROUTING_PARAMS_DEFAULT, proc_sm=proc_sm, proc_pet=proc_pet,
                  hourly=hourly, kind=kind)
    q_ora, tro_ora, qm_ora = o.run(forcing, 1, 1, n_steps, want_tro=True, want_qmod=True)
    return (q_gpu, np.concatenate(tros), np.concatenate(qms), st_gpu), (q_ora, tro_ora, qm_ora, o.state)


@pytest.fixture(scope="module")
def small():
    dom = synth.make_domain(24, 32, 3, 4, seed=1)
    p = synth.make_eff_params(dom, seed=3)
    f = synth.make_forcing(dom, 24 * 45, seed=2)
    return dom, p, f


def _assert_all_bitwise(gpu, ora):
    q_g, tro_g, qm_g, st_g = gpu
    q_o, tro_o, qm_o, st_o = ora
    assert bitwise(tro_g, tro_o), f"total runoff max rel {max_rel(tro_g, tro_o)}"
    assert bitwise(qm_g, qm_o), f"Qmod max rel {max_rel(qm_g, qm_o)}"
    assert bitwise(q_g, q_o), f"gauge Q max rel {max_rel(q_g, q_o)}"
    for k, ko in STATE_MAP.items():
        assert bitwise(st_g[k], st_o[ko]), f"state {k}: max rel {max_rel(st_g[k], st_o[ko])}"


def test_plain_hourly_bitwise(small):
    dom, p, f = small
    gpu, ora = run_pair(dom, p, f, 24 * 45)
    assert np.all(np.isfinite(gpu[0])) and gpu[0].max() > 0
    _assert_all_bitwise(gpu, ora)


def test_chunked_calls_bitwise(small):
    dom, p, f = small
    gpu, ora = run_pair(dom, p, f, 24 * 45, chunks=4)
    _assert_all_bitwise(gpu, ora)


@pytest.mark.parametrize("proc_sm", [2, 3, 4])
def test_soil_moisture_cases_bitwise(small, proc_sm):
    dom, p, f = small
    gpu, ora = run_pair(dom, p, f, 24 * 20, proc_sm=proc_sm)
    _assert_all_bitwise(gpu, ora)


@pytest.mark.parametrize("H", [1, 2, 6, 8])
def test_horizons_bitwise(H):
    dom = synth.make_domain(16, 20, H, 4, seed=5)
    p = synth.make_eff_params(dom, seed=6)
    f = synth.make_forcing(dom, 24 * 15, seed=7)
    gpu, ora = run_pair(dom, p, f, 24 * 15)
    _assert_all_bitwise(gpu, ora)


def test_pet_lai_correction_bitwise(small):
    dom, p, f = small
    gpu, ora = run_pair(dom, p, f, 24 * 20, proc_pet=-1)
    _assert_all_bitwise(gpu, ora)


def test_against_libm_oracle(small):
    """Reference semantics (C library exp/log/pow): 1e-9 relative."""
    dom, p, f = small
    gpu, ora = run_pair(dom, p, f, 24 * 45, kind="libm")
    q_g, tro_g, qm_g, st_g = gpu
    q_o, tro_o, qm_o, st_o = ora
    assert max_rel(q_g, q_o) <= 1e-9
    for k, ko in STATE_MAP.items():
        assert max_rel(st_g[k], st_o[ko]) <= 1e-9, k


def test_daily_forcing_hargreaves():
    """Daily forcing at hourly steps (day/night disaggregation) with
    Hargreaves-Samani PET; CUDA trig for the radiation term: 1e-12 relative."""
    dom = synth.make_domain(16, 24, 3, 4, seed=11)
    p = synth.make_eff_params(dom, seed=12)
    fd = synth.make_daily_forcing(dom, 30, seed=13)
    forcing = {"pre": fd["pre"], "temp": fd["temp"], "tmin": fd["tmin"], "tmax": fd["tmax"]}
    gpu, ora = run_pair(dom, p, forcing, 24 * 30, proc_pet=1, hourly=False)
    q_g, tro_g, qm_g, st_g = gpu
    q_o, tro_o, qm_o, st_o = ora
    assert max_rel(q_g, q_o) <= 1e-12
    for k, ko in STATE_MAP.items():
        assert max_rel(st_g[k], st_o[ko]) <= 1e-12, k


def test_daily_forcing_pet_input_bitwise():
    """Daily forcing, PET input with aspect correction: all-hmath, bitwise."""
    dom = synth.make_domain(16, 24, 3, 4, seed=21)
    p = synth.make_eff_params(dom, seed=22)
    fd = synth.make_daily_forcing(dom, 20, seed=23)
    forcing = {"pre": fd["pre"], "temp": fd["temp"], "pet": fd["pet"]}
    gpu, ora = run_pair(dom, p, forcing, 24 * 20, proc_pet=0, hourly=False)
    _assert_all_bitwise(gpu, ora)


def test_members_independent(small):
    """Three parameter sets in one context equal three single runs, bitwise."""
    dom, _, f = small
    plist = [synth.make_eff_params(dom, seed=s) for s in (31, 32, 33)]
    rlist = np.array([synth.ROUTING_PARAMS_DEFAULT,
                      [0.33, 0.072, 2.05, 0.095, 0.2],
                      [0.315, 0.078, 1.97, 0.105, 0.45]])
    n = 24 * 10
    g = MhmGpu(dom, n_members=3)
    g.prepare(plist, rlist)
    g.set_meteo(1, **f)
    q3 = g.run(1, n)
    for m in range(3):
        s = MhmGpu(dom)
        s.prepare(plist[m], rlist[m])
        s.set_meteo(1, **f)
        q1 = s.run(1, n)
        assert bitwise(q3[m], q1[0])
        st3, st1 = g.get_state(m), s.get_state()
        for k in st1:
            assert bitwise(st3[k], st1[k]), k


def test_restart_roundtrip(small):
    """Stop, read the restart state, continue in a new context with
    read_states: identical to an uninterrupted run."""
    dom, p, f = small
    n1, n2 = 24 * 10, 24 * 12
    a = MhmGpu(dom)
    a.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
    a.set_meteo(1, **f)
    q_full = a.run(1, n1 + n2)
    b = MhmGpu(dom)
    b.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
    b.set_meteo(1, **f)
    b.run(1, n1)
    st = b.get_state()
    c = MhmGpu(dom, read_states=True)
    c.set_eff_params(p)
    c.set_state(st)
    c.set_meteo(1, **f)
    q2 = c.run(n1 + 1, n2)
    assert bitwise(q2[0], q_full[0][:, n1:])
    sa, sc = a.get_state(), c.get_state()
    for k in sa:
        assert bitwise(sa[k], sc[k]), k


def test_internal_chunking(monkeypatch, small):
    """A small device budget forces many internal chunks: same bits."""
    dom, p, f = small
    monkeypatch.setenv("MHM_CHUNK_BYTES", str(dom.n_cells * 8 * 37))
    gpu, ora = run_pair(dom, p, f, 24 * 12)
    _assert_all_bitwise(gpu, ora)


def test_device_forcing(small):
    torch = pytest.importorskip("torch")
    dom, p, f = small
    n = 24 * 10
    a = MhmGpu(dom)
    a.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
    a.set_meteo(1, **f)
    qa = a.run(1, n)
    b = MhmGpu(dom)
    b.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
    dev = {k: torch.from_numpy(v[:n]).cuda() for k, v in f.items()}
    b.set_meteo(1, dev["pre"], dev["temp"], dev["pet"], on_device=True)
    qb = b.run(1, n)
    assert bitwise(qa, qb)


@pytest.mark.parametrize("proc_sm", [1, 3])
def test_degenerate_parameters_bitwise(proc_sm):
    """Parameters at the edges the branches and divisions must handle like the
    reference: no / full sealing, zero sealed storage capacity (the huge()
    evaporation path), zero interception capacity in some months, field
    capacity or saturation equal to the wilting point (a zero stress
    denominator: IEEE division by zero), karstic gain (karstLoss > 1) and a
    zero Jarvis threshold."""
    dom = synth.make_domain(16, 20, 3, 4, seed=31)
    N, H = dom.n_cells, dom.n_horizons
    p = {k: np.array(v, np.float64, copy=True) for k, v in synth.make_eff_params(dom, seed=32).items()
         if v is not None}
    rng = np.random.default_rng(33)
    pick = lambda frac: rng.random(N) < frac   # noqa: E731
    p["fSealed"][pick(0.2)] = 0.0
    p["fSealed"][pick(0.1)] = 1.0
    p["sealedThresh"][pick(0.3)] = 0.0
    mi = p["maxInter"].reshape(12, N)
    mi[:, pick(0.2)] = 0.0
    for name in ("soilMoistFC", "soilMoistSat"):
        a = p[name].reshape(H, N)
        sel = pick(0.15)
        a[1, sel] = p["wiltingPoint"].reshape(H, N)[1, sel]
    p["karstLoss"][pick(0.2)] = 1.05
    if "jarvis_thresh_c1" in p:
        p["jarvis_thresh_c1"][pick(0.3)] = 0.0
    else:
        p["jarvis_thresh_c1"] = np.where(pick(0.3), 0.0, 0.5)
    f = synth.make_forcing(dom, 24 * 20, seed=34, gamma_theta=4.0)
    gpu, ora = run_pair(dom, p, f, 24 * 20, proc_sm=proc_sm)
    _assert_all_bitwise(gpu, ora)


@pytest.mark.parametrize("H", [3, 6])
def test_unbounded_runoff_fraction_bitwise(H):
    """The warp evaluates the horizons' runoff fractions exp(beta log(SM/SMs))
    only for cells with effective precipitation other than +0, unless a
    cell's fraction may leave [0, 1]: beta zero, negative or subnormal, SMs
    infinite.  Cells with those parameters, mixed with ordinary ones in every
    warp, under forcing with 70 % dry hours, equal the oracle bit for bit."""
    dom = synth.make_domain(16, 20, H, 4, seed=41)
    N = dom.n_cells
    p = {k: np.array(v, np.float64, copy=True) for k, v in synth.make_eff_params(dom, seed=42).items()
         if v is not None}
    rng = np.random.default_rng(43)
    cat = rng.integers(0, 5, N)          # 0 ordinary, 1 beta = 0, 2 beta < 0, 3 beta subnormal, 4 SMs = inf
    beta = p["soilMoistExp"].reshape(H, N)
    sms = p["soilMoistSat"].reshape(H, N)
    for h in (0, H - 1):
        beta[h, cat == 1] = 0.0
        beta[h, cat == 2] = -0.4
        beta[h, cat == 3] = 5e-324
        sms[h, cat == 4] = np.inf
    f = synth.make_forcing(dom, 24 * 20, seed=44)
    gpu, ora = run_pair(dom, p, f, 24 * 20)
    _assert_all_bitwise(gpu, ora)


def test_members_across_warps_bitwise():
    """Three parameter sets on 255 cells and 6 horizons: warps hold the last
    cells of one member and the first of the next, and the packed runoff
    fractions read the other lanes' parameter planes.  Each member equals
    its own oracle run bit for bit."""
    dom = synth.make_domain(15, 17, 6, 3, seed=51)
    plist = [synth.make_eff_params(dom, seed=s) for s in (52, 53, 54)]
    rlist = np.array([synth.ROUTING_PARAMS_DEFAULT,
                      [0.33, 0.072, 2.05, 0.095, 0.2],
                      [0.315, 0.078, 1.97, 0.105, 0.45]])
    f = synth.make_forcing(dom, 24 * 12, seed=55)
    n = 24 * 12
    g = MhmGpu(dom, n_members=3)
    g.prepare(plist, rlist)
    g.set_meteo(1, **f)
    q3 = g.run(1, n)
    for m in range(3):
        o = OracleRun(dom, plist[m], rlist[m])
        q_o, _, _ = o.run(f, 1, 1, n)
        assert bitwise(q3[m].T, q_o), f"member {m}: gauge Q max rel {max_rel(q3[m].T, q_o)}"
        st = g.get_state(m)
        for k, ko in STATE_MAP.items():
            assert bitwise(st[k], o.state[ko]), f"member {m} state {k}: max rel {max_rel(st[k], o.state[ko])}"
