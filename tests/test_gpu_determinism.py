"""Determinism: the same input run twice gives bit-identical output on every
launch path -- the cell chain in both thread mappings (one member per block;
member-tiled blocks), MPR of many members, routing by per-tick graph and by
cluster walk, and the fused multi-context launch whose blocks take tiles
from a device counter in whatever order they reach it (no result depends
on that order: each work item's arithmetic is its own)."""
import numpy as np
import pytest

from mhm_gb300 import params, synth

pytestmark = pytest.mark.gpu


def _ensemble_run(cluster: str, monkeypatch):
    from mhm_gb300.model import MhmGpu
    monkeypatch.setenv("MHM_ROUTE_CLUSTER", cluster)
    dom = synth.make_domain(36, 30, 3, l11_factor=3, seed=12, dem_kind="fractal", ridges=1)
    l0 = synth.make_l0(dom, 2, seed=13)
    gam = params.random_gammas(12, 1, 0, 1, l0.n_geo, seed=14)   # 12 members: member-tiled blocks
    f = synth.make_forcing(dom, 120, seed=15)
    g = MhmGpu(dom, n_members=12)
    try:
        g.mpr_setup(l0)
        g.mpr(gam)
        p = [g.get_eff_params(m) for m in (0, 11)]
        for m in range(12):
            g.init_states(m)
        g.set_meteo(1, **f)
        q = np.concatenate([g.run(1, 60), g.run(61, 60)], axis=2)
        st = [g.get_state(m) for m in (0, 5, 11)]
    finally:
        g.close()
    return q, st, p


@pytest.mark.parametrize("cluster", ["0", "8"])
def test_same_input_same_bits(cluster, monkeypatch):
    qa, sa, pa = _ensemble_run(cluster, monkeypatch)
    qb, sb, pb = _ensemble_run(cluster, monkeypatch)
    assert np.all(np.isfinite(qa))
    assert np.array_equal(qa.view(np.uint64), qb.view(np.uint64))
    for x, y in zip(sa, sb):
        for k in x:
            assert np.array_equal(np.asarray(x[k]).view(np.uint64), np.asarray(y[k]).view(np.uint64)), k
    for x, y in zip(pa, pb):
        for k in x:
            assert np.array_equal(x[k], y[k]), k


def test_fused_launch_is_deterministic():
    import torch
    from mhm_gb300.model import MhmBatch, MhmGpu
    C = 48

    def run():
        ctxs, qs = [], []
        for i, (nr, nc, H, M) in enumerate([(30, 28, 6, 2), (12, 10, 2, 4), (20, 24, 4, 1)]):
            dom = synth.make_domain(nr, nc, H, l11_factor=2, seed=70 + i)
            l0 = synth.make_l0(dom, 2, seed=80 + i)
            g = MhmGpu(dom, n_members=M)
            g.mpr_setup(l0)
            g.mpr(params.random_gammas(M, 1, 0, 1, l0.n_geo, seed=90 + i))
            for m in range(M):
                g.init_states(m)
            f = synth.make_forcing(dom, C, seed=95 + i)
            g.set_meteo(1, *[torch.from_numpy(f[k]).cuda() for k in ("pre", "temp", "pet")], on_device=True)
            ctxs.append(g)
        batch = MhmBatch()
        try:
            for r in range(3):
                q = [np.zeros((g.n_members, 1, C)) for g in ctxs]
                batch.run_members(ctxs, [np.full(g.n_members, 1 + r * C, np.int32) for g in ctxs], C, q)
                for g in ctxs:
                    g.sync()
                qs.append(q)
            st = [g.get_state(0) for g in ctxs]
        finally:
            batch.close()
            for g in ctxs:
                g.close()
        return qs, st

    qa, sa = run()
    qb, sb = run()
    for ra, rb in zip(qa, qb):
        for x, y in zip(ra, rb):
            assert np.array_equal(x.view(np.uint64), y.view(np.uint64))
    for x, y in zip(sa, sb):
        for k in x:
            assert np.array_equal(x[k], y[k]), k
