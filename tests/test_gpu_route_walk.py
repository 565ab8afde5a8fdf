"""The routing wavefront of a chunk walked in one launch by thread-block
clusters (route_cluster 4, 8, 16) gives the discharge and routing states of
the per-tick launches bit for bit -- over several chunks and calls, with more
members than resident clusters (each cluster then walks several members),
with idle members (member mode), with inflow gauges that cut a link, and with
the adaptive routing step of routing case 2 -- and the gauge discharge of the
oracle's sequential L11_routing (src/mRM/mo_mrm_routing.f90:380-481)."""
import numpy as np
import pytest

from mhm_gb300 import synth

pytestmark = pytest.mark.gpu

ROUT_KEYS = ("qOUT", "Qmod", "qTIN", "qTR")


def _chunked(monkeypatch, cluster: int, dom, n_members: int, steps: int = 40):
    monkeypatch.setenv("MHM_ROUTE_CLUSTER", str(cluster))
    monkeypatch.setenv("MHM_CHUNK_BYTES", str(2 * n_members * dom.n_cells * 8 * steps))


def _run_plain(monkeypatch, cluster: int, n_members: int = 2):
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(48, 48, 3, l11_factor=2, seed=4)
    _chunked(monkeypatch, cluster, dom, n_members)
    ps = [synth.make_eff_params(dom, seed=3 + m) for m in range(n_members)]
    f = synth.make_forcing(dom, 200, seed=2)
    g = MhmGpu(dom, n_members=n_members)
    try:
        assert g.get_launch_config()["route_cluster"] == cluster
        g.prepare(ps, synth.ROUTING_PARAMS_DEFAULT)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        q = [g.run(1, 100), g.run(101, 37), g.run(138, 63)]
        st = [g.get_state(m) for m in range(n_members)]
    finally:
        g.close()
    return np.concatenate(q, axis=2), st


@pytest.mark.parametrize("cluster", [4, 8, 16])
def test_walk_equals_tick_launches(monkeypatch, cluster):
    qa, sa = _run_plain(monkeypatch, 0)
    qb, sb = _run_plain(monkeypatch, cluster)
    assert np.array_equal(qa, qb)
    for a, b in zip(sa, sb):
        for k in ROUT_KEYS:
            assert np.array_equal(a[k], b[k]), k


def test_walk_with_more_members_than_clusters(monkeypatch):
    """40 members on 16-CTA clusters (fewer can be resident than members):
    each cluster walks members c, c + n_clusters, ..."""
    qa, sa = _run_plain(monkeypatch, 0, n_members=40)
    qb, sb = _run_plain(monkeypatch, 16, n_members=40)
    assert np.array_equal(qa, qb)
    for a, b in zip(sa, sb):
        for k in ROUT_KEYS:
            assert np.array_equal(a[k], b[k]), k


def _run_members(monkeypatch, cluster: int):
    """member mode: members at different steps, one idle member per call"""
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(32, 28, 2, l11_factor=2, seed=6)
    _chunked(monkeypatch, cluster, dom, 4, steps=48)
    ps = [synth.make_eff_params(dom, seed=10 + m) for m in range(4)]
    f = synth.make_forcing(dom, 96, seed=7)
    g = MhmGpu(dom, n_members=4)
    try:
        g.prepare(ps, synth.ROUTING_PARAMS_DEFAULT)
        import torch
        dev = {k: torch.from_numpy(np.ascontiguousarray(f[k])).cuda() for k in ("pre", "temp", "pet")}
        g.set_meteo(1, dev["pre"], dev["temp"], dev["pet"], on_device=True)
        qs = []
        for t0 in ([1, 25, -1, 49], [-1, 73, 97, 121]):
            q = np.zeros((4, len(dom.gauge_node), 48))
            g.run_members_async(t0, 48, q)
            g.sync()
            qs.append(q)
        st = [g.get_state(m) for m in range(4)]
    finally:
        g.close()
    return qs, st


@pytest.mark.parametrize("cluster", [8])
def test_walk_member_mode(monkeypatch, cluster):
    qa, sa = _run_members(monkeypatch, 0)
    qb, sb = _run_members(monkeypatch, cluster)
    for a, b in zip(qa, qb):
        assert np.array_equal(a, b)
    for a, b in zip(sa, sb):
        for k in ROUT_KEYS:
            assert np.array_equal(a[k], b[k]), k


def test_walk_against_oracle(monkeypatch):
    """gauge discharge of a 2-member run walked by 8-CTA clusters equals the
    oracle's sequential routing of each member, bit for bit"""
    from mhm_gb300.model import MhmGpu
    from oracle import oracle
    dom = synth.make_domain(40, 36, 3, l11_factor=2, seed=9, dem_kind="fractal", ridges=1)
    _chunked(monkeypatch, 8, dom, 2, steps=60)
    ps = [synth.make_eff_params(dom, seed=20 + m) for m in range(2)]
    T = 150
    f = synth.make_forcing(dom, T, seed=3)
    g = MhmGpu(dom, n_members=2)
    try:
        g.prepare(ps, synth.ROUTING_PARAMS_DEFAULT)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        q = g.run(1, T)
    finally:
        g.close()
    for m in range(2):
        run = oracle.OracleRun(dom, ps[m], rout_param=synth.ROUTING_PARAMS_DEFAULT, kind="hmath")
        qo = run.run(f, 1, 1, T)[0]
        assert np.array_equal(q[m].T, qo), m
