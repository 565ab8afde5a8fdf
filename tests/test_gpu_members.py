"""Members at their own model steps (continuous batching) and device-resident
restart snapshots.

A member admitted into a running batch at a later chunk, or left idle, must
produce exactly what the same run gives alone through the ordinary mhm_run
path (same warm-start states, same forcing rows, same calendar)."""
import numpy as np
import pytest

from mhm_gb300 import params, synth

pytestmark = pytest.mark.gpu

C = 24  # steps per chunk


def _setup():
    import torch
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(16, 12, 3, l11_factor=2, seed=1)
    l0 = synth.make_l0(dom, 2, seed=4)
    gam = params.random_gammas(4, 1, 0, 1, l0.n_geo, seed=7)
    f = synth.make_forcing(dom, C, seed=2)
    win = [torch.from_numpy(f[k]).cuda() for k in ("pre", "temp", "pet")]
    # spin-up from default states (45 days) -> the warm-start restart
    s = MhmGpu(dom, n_members=1)
    s.mpr_setup(l0)
    s.mpr(params.default_gamma(1, 0, 1, l0.n_geo))
    s.init_states(0)
    for c in range(45):
        s.set_meteo(1 + c * C, *win, on_device=True)
        s.run(1 + c * C, C)
    # states only: each run keeps the Muskingum coefficients of its own parameters
    restart = {k: v for k, v in s.get_state(0).items() if k not in ("C1", "C2")}
    s.close()
    return dom, l0, gam, win, restart


def test_members_at_own_steps_equal_runs_alone():
    from mhm_gb300.model import MhmGpu
    dom, l0, gam, win, restart = _setup()
    G = len(dom.gauge_node)
    # schedule: start chunk and number of chunks of each member (member 2 idle at first)
    start = [0, 1, 3, 0]
    length = [4, 3, 2, 2]
    n_chunks = 5
    mix = MhmGpu(dom, n_members=4, read_states=True)
    try:
        mix.mpr_setup(l0)
        mix.mpr(gam)
        mix.snapshot_alloc(1)
        mix.set_state(restart, 0)
        mix.snapshot_save(0, 0)
        q_mix = {m: [] for m in range(4)}
        for c in range(n_chunks):
            tt0 = np.zeros(4, np.int32)
            for m in range(4):
                if start[m] == c:
                    mix.snapshot_load(0, m)            # warm start on admission
                if start[m] <= c < start[m] + length[m]:
                    tt0[m] = 1 + (c - start[m]) * C
            mix.set_meteo(1, *win, on_device=True)
            q = np.zeros((4, G, C))
            mix.run_members_async(tt0, C, q)
            mix.sync()
            for m in range(4):
                if tt0[m] > 0:
                    q_mix[m].append(q[m].copy())
                else:
                    assert np.all(q[m] == 0.0)              # idle slot: no discharge
        st_mix = {m: mix.get_state(m) for m in range(4)}
    finally:
        mix.close()
    for m in range(4):
        alone = MhmGpu(dom, n_members=1, read_states=True)
        try:
            alone.mpr_setup(l0)
            alone.mpr(gam[m])
            alone.set_state(restart, 0)
            qa = []
            for c in range(length[m]):
                tt0 = 1 + c * C
                alone.set_meteo(tt0, *win, on_device=True)
                qa.append(alone.run(tt0, C)[0])
            st = alone.get_state(0)
        finally:
            alone.close()
        assert len(qa) == len(q_mix[m])
        for a, b in zip(qa, q_mix[m]):
            assert np.array_equal(a, b), m
        for k in ("interc", "snowpack", "soilMoist", "unsatSTW", "satSTW", "qTR", "qTIN"):
            assert np.array_equal(st[k], st_mix[m][k]), (m, k)


def test_snapshot_roundtrip_restores_states():
    from mhm_gb300.model import MhmGpu
    dom, l0, gam, win, restart = _setup()
    g = MhmGpu(dom, n_members=2, read_states=True)
    try:
        g.mpr_setup(l0)
        g.mpr(gam[:2])
        g.snapshot_alloc(2)
        g.set_state(restart, 1)
        g.snapshot_save(1, 1)
        g.set_meteo(1, *win, on_device=True)
        g.run_members_async(np.array([0, 1], np.int32), C)   # member 1 moves on
        g.sync()
        assert not np.array_equal(g.get_state(1)["soilMoist"], restart["soilMoist"])
        g.snapshot_load(1, 1)
        back = g.get_state(1)
        for k in ("interc", "snowpack", "sealSTW", "soilMoist", "unsatSTW", "satSTW", "qTIN", "qTR", "qOUT"):
            assert np.array_equal(back[k], restart[k]), k
    finally:
        g.close()
