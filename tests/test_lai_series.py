"""Gridded LAI series (timeStep_LAI_input -1 / -2 / -3).

CPU: the library's closed-form LAI index (mhm_step_lai: days / months /
years counted from the run's first step) equals the oracle's literal
restatement of datetimeinfo_update_LAI_timestep (a counter raised on the
increment's is_new_day / month / year flags,
src/common/mo_common_datetime_type.f90:138-155) for many start dates, time
steps and all modes.
GPU: runs with a series -- chunked calls, per-member steps, PET cases 0 and
-1 -- equal the oracle's time loop bit for bit, and a run beyond the series
is refused."""
import ctypes as C

import numpy as np
import pytest

from mhm_gb300 import synth

_ip = C.POINTER(C.c_int32)


@pytest.mark.parametrize("jul_start", [2447894, 2448257, 2451545 + 59, 2440588])
@pytest.mark.parametrize("timestep", [1, 6, 24])
@pytest.mark.parametrize("mode", [0, -1, -2, -3])
def test_lai_index_equals_the_reference_counter(jul_start, timestep, mode, lib, ora_hmath):
    n = max((24 // timestep) * 500, 600)
    got = np.zeros(n, np.int32)
    assert lib.mhm_step_lai(jul_start, timestep, mode, 1, n, got.ctypes.data_as(_ip)) == 0
    want = np.zeros(n, np.int32)
    ora_hmath.ora_step_lai(jul_start, timestep, mode, n, want.ctypes.data_as(_ip))
    assert np.array_equal(got, want)
    # a later first step gives the same indexes (chunked runs)
    part = np.zeros(100, np.int32)
    assert lib.mhm_step_lai(jul_start, timestep, mode, 501, 100, part.ctypes.data_as(_ip)) == 0
    assert np.array_equal(part, want[500:600])


def _series(dom, n_lai, seed):
    rng = np.random.default_rng(seed)
    N = dom.n_cells
    return (rng.uniform(0.05, 3.0, (n_lai, N)), rng.uniform(0.7, 1.3, (n_lai, N)))


@pytest.mark.gpu
@pytest.mark.parametrize("mode,n_lai,proc_pet", [(-2, 3, 0), (-1, 9, -1), (-3, 1, 0)])
def test_gpu_series_equals_oracle(mode, n_lai, proc_pet):
    from mhm_gb300.model import MhmGpu
    from oracle import oracle
    dom = synth.make_domain(20, 18, 3, l11_factor=2, seed=31, jul_start=2447919)   # 1990-01-27
    p = synth.make_eff_params(dom, seed=32)
    T = 24 * 8 if mode == -1 else 24 * 40
    f = synth.make_forcing(dom, T, seed=33)
    mi, pl = _series(dom, n_lai, 34)
    g = MhmGpu(dom, proc_pet=proc_pet)
    try:
        g.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
        g.set_lai_series(mode, n_lai)
        g.set_lai_params(mi, pl if proc_pet == -1 else None)
        g.set_meteo(1, **f)
        q = np.concatenate([g.run(1, T // 2), g.run(T // 2 + 1, T - T // 2)], axis=2)[0].T
        st = g.get_state()
    finally:
        g.close()
    po = dict(p)
    po["maxInter"] = mi.reshape(-1)
    if proc_pet == -1:
        po["petLAIcorFactor"] = pl.reshape(-1)
    run = oracle.OracleRun(dom, po, rout_param=synth.ROUTING_PARAMS_DEFAULT, proc_pet=proc_pet, kind="hmath",
                           lai_mode=mode, n_lai=n_lai)
    qo = run.run(f, 1, 1, T)[0]
    assert np.array_equal(q.view(np.uint64), qo.view(np.uint64))
    assert np.array_equal(st["interc"], run.state["interc"])
    # the LAI entries matter: monthly slots give another result
    g2 = MhmGpu(dom, proc_pet=proc_pet)
    try:
        g2.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
        g2.set_meteo(1, **f)
        q2 = g2.run(1, T)[0].T
    finally:
        g2.close()
    assert not np.array_equal(q2, q)


@pytest.mark.gpu
def test_gpu_series_must_cover_the_run():
    from mhm_gb300.model import MhmError, MhmGpu
    dom = synth.make_domain(10, 8, 2, l11_factor=2, seed=3, jul_start=2447893)     # 1990-01-01
    p = synth.make_eff_params(dom, seed=4)
    f = synth.make_forcing(dom, 24 * 40, seed=5)
    g = MhmGpu(dom)
    try:
        g.prepare(p, synth.ROUTING_PARAMS_DEFAULT)
        g.set_lai_series(-2, 1)                      # January only
        g.set_lai_params(_series(dom, 1, 6)[0])
        g.set_meteo(1, **f)
        g.run(1, 24 * 31)                            # January: fine
        with pytest.raises(MhmError):
            g.run(24 * 31 + 1, 24)                   # February 1st needs entry 2
    finally:
        g.close()


@pytest.mark.gpu
def test_gpu_series_in_member_mode():
    """members at their own steps read the series entry of their own date"""
    import torch
    from mhm_gb300.model import MhmGpu
    from oracle import oracle
    dom = synth.make_domain(14, 12, 2, l11_factor=2, seed=41, jul_start=2447950)   # 1990-02-27
    ps = [synth.make_eff_params(dom, seed=42 + m) for m in range(2)]
    C_ = 48
    f = synth.make_forcing(dom, C_, seed=44)
    n_lai = 4
    mis = [_series(dom, n_lai, 45 + m)[0] for m in range(2)]
    g = MhmGpu(dom, n_members=2)
    try:
        g.prepare(ps, synth.ROUTING_PARAMS_DEFAULT)
        g.set_lai_series(-2, n_lai)
        for m in range(2):
            g.set_lai_params(mis[m], member=m)
        g.set_meteo(1, *[torch.from_numpy(f[k]).cuda() for k in ("pre", "temp", "pet")], on_device=True)
        q = np.zeros((2, 1, C_))
        g.run_members_async(np.array([1, 24 * 40 + 1], np.int32), C_, q)   # member 1 starts in April
        g.sync()
    finally:
        g.close()
    for m, t0 in ((0, 1), (1, 24 * 40 + 1)):
        po = dict(ps[m])
        po["maxInter"] = mis[m].reshape(-1)
        run = oracle.OracleRun(dom, po, rout_param=synth.ROUTING_PARAMS_DEFAULT, kind="hmath", lai_mode=-2,
                               n_lai=n_lai)
        qo = run.run(f, t0, t0, C_)[0][:, 0]       # the window's rows from the member's own step
        assert np.array_equal(q[m, 0].view(np.uint64), qo.view(np.uint64)), m


@pytest.mark.gpu
@pytest.mark.parametrize("proc_pet", [0, -1])
def test_gpu_mpr_of_a_gridded_series_and_its_run(proc_pet):
    """mpr() over a gridded L0 LAI series of 15 monthly entries writes the
    series' maxInter (and LAI correction factors) equal to the oracle's mpr()
    over the same entries, and the run with them equals the oracle's"""
    from mhm_gb300 import params
    from mhm_gb300.model import MhmGpu
    from oracle import oracle
    dom = synth.make_domain(16, 14, 3, l11_factor=2, seed=51, jul_start=2447893)     # 1990-01-01
    l0 = synth.make_l0(dom, 2, seed=52)
    n_lai = 15
    l0.lai_series = np.random.default_rng(53).uniform(0.2, 6.0, (n_lai, l0.n_cells0))
    l0.gridded_lai = True
    gam = params.random_gammas(2, 1, proc_pet, 1, l0.n_geo, seed=54)
    off = params.offsets(1, proc_pet, 1, l0.n_geo)
    T = 24 * 45
    f = synth.make_forcing(dom, T, seed=55)
    g = MhmGpu(dom, proc_pet=proc_pet, n_members=2)
    try:
        g.set_lai_series(-2, n_lai)
        g.mpr_setup(l0)
        g.mpr(gam)
        series = [g.get_lai_params(n_lai, m) for m in range(2)]
        p_dev = [g.get_eff_params(m) for m in range(2)]
        for m in range(2):
            g.init_states(m)
        g.set_meteo(1, **f)
        q = g.run(1, T)
    finally:
        g.close()
    for m in range(2):
        po = oracle.oracle_mpr(dom.n_cells, 3, l0, gam[m], off, 1, proc_pet, "hmath")
        assert np.array_equal(series[m][0].reshape(-1), po["maxInter"]), m
        if proc_pet == -1:
            assert np.array_equal(series[m][1].reshape(-1), po["petLAIcorFactor"]), m
        p = {k: v for k, v in p_dev[m].items()}
        p["maxInter"] = series[m][0].reshape(-1)
        p["petLAIcorFactor"] = series[m][1].reshape(-1)
        run = oracle.OracleRun(dom, p, rout_param=gam[m][off[7]:off[7] + 5], proc_pet=proc_pet, kind="hmath",
                               lai_mode=-2, n_lai=n_lai)
        qo = run.run(f, 1, 1, T)[0][:, 0]
        assert np.array_equal(q[m, 0].view(np.uint64), qo.view(np.uint64)), m


@pytest.mark.gpu
def test_gpu_series_in_a_fused_launch():
    """a context with a gridded LAI series and one with monthly slots, their
    cell chains in one fused launch, equal the same calls made one context at
    a time"""
    import torch
    from mhm_gb300.model import MhmBatch, MhmGpu
    C_ = 48

    def contexts():
        out = []
        for i, series in enumerate((True, False)):
            dom = synth.make_domain(14 + 2 * i, 12, 2 + i, l11_factor=2, seed=61 + i, jul_start=2447950)
            p = synth.make_eff_params(dom, seed=62 + i)
            g = MhmGpu(dom, n_members=2)
            g.prepare([p, p], synth.ROUTING_PARAMS_DEFAULT)
            if series:
                g.set_lai_series(-1, 4)                      # daily entries
                for m in range(2):
                    g.set_lai_params(_series(dom, 4, 63 + m)[0], member=m)
            f = synth.make_forcing(dom, C_, seed=64 + i)
            g.set_meteo(1, *[torch.from_numpy(f[k]).cuda() for k in ("pre", "temp", "pet")], on_device=True)
            out.append(g)
        return out

    ref, fused = contexts(), contexts()
    batch = MhmBatch()
    try:
        t0 = [np.array([1, 25], np.int32), np.array([1, 0], np.int32)]
        qa = [np.zeros((2, 1, C_)) for _ in ref]
        qb = [np.zeros((2, 1, C_)) for _ in fused]
        for g, t, q in zip(ref, t0, qa):
            g.run_members_async(t, C_, q)
            g.sync()
        batch.run_members(fused, t0, C_, qb)
        for g in fused:
            g.sync()
        for x, y in zip(qa, qb):
            assert np.array_equal(x.view(np.uint64), y.view(np.uint64))
    finally:
        batch.close()
        for g in ref + fused:
            g.close()
