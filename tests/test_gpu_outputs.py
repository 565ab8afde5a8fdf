"""Aggregated flux/state outputs (outputFlxState) and mRM's Qrouted on the
device against the oracle, bit for bit: every variable, per-horizon planes,
intervals of n steps / a day / a month / the whole run / none, warm-up,
several chunks per run call and several run calls, the next-scene weights of
one step, two members, and Qrouted with a multi-step routing window.  Plus
the refusals that need no device work."""
import numpy as np
import pytest

from mhm_gb300 import outputs, synth
from oracle import oracle

ALL = [1 if i != 18 else 0 for i in range(1, 22)]      # every variable but neutrons


def _run_both(monkeypatch, interval, interval_mrm, warm, calls, proc_rout=1, cellsize=1000.0, l11=2, weights_at=0,
              chunk_steps=None, flags=ALL):
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(10, 12, 3, l11_factor=l11, seed=5, cellsize_m=cellsize)
    N, H = dom.n_cells, dom.n_horizons
    M = 2
    ps = [synth.make_eff_params(dom, seed=3 + m) for m in range(M)]
    rp = [1.5, 0, 0, 0, 0] if proc_rout == 2 else list(synth.ROUTING_PARAMS_DEFAULT)
    T = sum(calls)
    f = synth.make_forcing(dom, T, seed=2, gamma_theta=4.0)
    w_fs = [np.clip(p["fSealed"] * 0.5 + 0.1, 0.0, 1.0) for p in ps]
    w_sms = [np.asarray(p["soilMoistSat"]).reshape(H, N) * 1.1 for p in ps]
    if chunk_steps:
        monkeypatch.setenv("MHM_CHUNK_BYTES", str(2 * M * N * 8 * chunk_steps))
    g = MhmGpu(dom, proc_routing=proc_rout, n_members=M)
    try:
        g.prepare(ps, np.asarray(rp, np.float64))
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        g.enable_flux_state_outputs(flags, interval, warm, T, max_slots=T)
        g.enable_routed_outputs(interval_mrm, warm, T, max_slots=T)
        if weights_at:
            for m in range(M):
                g.set_output_weights(m, weights_at, w_fs[m], w_sms[m])
        tt = 1
        for n in calls:
            g.run(tt, n)
            tt += n
        names, fs, fs_tt = g.read_flux_state_outputs()
        qr, qr_tt = g.read_routed_outputs()
    finally:
        g.close()
    for m in range(M):
        o = oracle.OracleRun(dom, ps[m], rout_param=rp, proc_rout=proc_rout)
        o.enable_outputs(interval, flags, warm, T, T, interval_mrm, True)
        if weights_at:
            o.set_output_weights(weights_at, w_fs[m], w_sms[m])
        tt = 1
        for n in calls:
            o.run(f, 1, tt, n)
            tt += n
        ofs, ofs_tt, oqr, oqr_tt = o.read_outputs()
        assert names == outputs.plane_names(flags, H)
        assert np.array_equal(fs_tt, ofs_tt) and np.array_equal(qr_tt, oqr_tt)
        assert fs.shape[:2] == ofs.shape[:2], (fs.shape, ofs.shape)
        for i, name in enumerate(names):
            assert np.array_equal(fs[:, i, m], ofs[:, i]), (m, name)
        assert np.array_equal(qr[:, m], oqr), m
    return names, fs, fs_tt, qr_tt


@pytest.mark.gpu
@pytest.mark.parametrize("interval", [-1, 7, 0])
def test_gpu_outputs_bitwise(monkeypatch, interval):
    names, fs, fs_tt, qr_tt = _run_both(monkeypatch, interval, -1, warm=30, calls=[100, 92], chunk_steps=45)
    assert len(names) == 16 + 4 * 3        # 16 single planes; SWC, SM, soil_infil, aET_L per horizon
    if interval == -1:
        assert list(fs_tt[:3]) == [48, 72, 96] and fs_tt[-1] == 192
    if interval == 7:
        assert list(fs_tt[:2]) == [37, 44]
    if interval == 0:
        assert list(fs_tt) == [192]
    assert list(qr_tt[:2]) == [48, 72]


@pytest.mark.gpu
def test_gpu_outputs_monthly_and_weights(monkeypatch):
    # Jan 2000 start: the month ends after step 744; next-scene weights at step 744
    _run_both(monkeypatch, -2, -2, warm=24, calls=[744, 96], weights_at=744, chunk_steps=300)


@pytest.mark.gpu
def test_gpu_outputs_none_written(monkeypatch):
    names, fs, fs_tt, qr_tt = _run_both(monkeypatch, -4, -4, warm=0, calls=[48], flags=[1, 0, 1] + [0] * 18)
    assert fs.shape[0] == 0 and qr_tt.size == 0


@pytest.mark.gpu
def test_gpu_qrouted_with_routing_windows(monkeypatch):
    # 3 km cells, L11 = 4 x 4 L1: routing step of 2 model steps (check case_09's adaptive routing)
    _run_both(monkeypatch, 5, 3, warm=10, calls=[48, 48], proc_rout=2, cellsize=3000.0, l11=4, chunk_steps=24)


@pytest.mark.gpu
def test_gpu_output_refusals():
    from mhm_gb300.model import MhmError, MhmGpu
    dom = synth.make_domain(6, 6, 2, l11_factor=2, seed=1)
    g = MhmGpu(dom, proc_routing=0)
    try:
        with pytest.raises(MhmError):
            g.enable_flux_state_outputs([18], 0, 0, 10)        # neutrons: process 10 not built
        with pytest.raises(MhmError):
            g.enable_routed_outputs(0, 0, 10)                  # no routing
        p = synth.make_eff_params(dom)
        g.prepare(p)
        f = synth.make_forcing(dom, 48)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        g.enable_flux_state_outputs([11], -1, 0, 48, max_slots=1)
        with pytest.raises(MhmError):
            g.run(1, 48)                                       # two days need two slots
        g.run(1, 24)
        names, fs, tt = g.read_flux_state_outputs()
        assert names == ["Q"] and list(tt) == [24]
        g.run(25, 24)                                          # the read freed the slot
    finally:
        g.close()
