"""The persistent multi-context launch (mhm_batch_run_members): basins of
different sizes and soil-horizon counts, each with its own members at their
own model steps, advanced chunk by chunk with the cell chains of all of them
in one launch per chunk from a device work queue.  Every context's discharge
and states must equal, bit for bit, the same calls made one context at a
time (mhm_run_members_async)."""
import numpy as np
import pytest

from mhm_gb300 import params, synth

pytestmark = pytest.mark.gpu

C = 48  # steps per chunk


def _basins():
    import torch
    out = []
    for i, (nr, nc, H, M) in enumerate([(40, 36, 6, 2), (9, 8, 2, 1), (24, 30, 3, 3), (16, 10, 5, 2)]):
        dom = synth.make_domain(nr, nc, H, l11_factor=2, seed=30 + i)
        l0 = synth.make_l0(dom, 2, seed=40 + i)
        gam = params.random_gammas(M, 1, 0, 1, l0.n_geo, seed=50 + i)
        f = synth.make_forcing(dom, C, seed=60 + i)
        win = [torch.from_numpy(f[k]).cuda() for k in ("pre", "temp", "pet")]
        out.append((dom, l0, gam, win, M))
    return out


def _contexts(basins):
    from mhm_gb300.model import MhmGpu
    ctxs = []
    for dom, l0, gam, win, M in basins:
        g = MhmGpu(dom, n_members=M)
        g.mpr_setup(l0)
        g.mpr(gam)
        for m in range(M):
            g.init_states(m)
        g.set_meteo(1, *win, on_device=True)
        ctxs.append(g)
    return ctxs


# member schedule per round: model step of each member (0: idle)
def _schedule(M, r):
    return np.array([1 + r * C if (m + r) % 3 != 2 else 0 for m in range(M)], np.int32)


def test_batch_equals_contexts_one_at_a_time():
    from mhm_gb300.model import MhmBatch
    basins = _basins()
    ref = _contexts(basins)
    fused = _contexts(basins)
    batch = MhmBatch()
    try:
        q_ref, q_fus = [], []
        for r in range(3):
            qa = [np.zeros((M, 1, C)) for *_, M in basins]
            qb = [np.zeros((M, 1, C)) for *_, M in basins]
            t0s = [_schedule(M, r) for *_, M in basins]
            for g, t0, q in zip(ref, t0s, qa):
                g.run_members_async(t0, C, q)
                g.sync()
            batch.run_members(fused, t0s, C, qb)
            for g in fused:
                g.sync()
            q_ref.append(qa)
            q_fus.append(qb)
        for r in range(3):
            for i in range(len(basins)):
                assert np.array_equal(q_ref[r][i].view(np.uint64), q_fus[r][i].view(np.uint64)), (r, i)
        for gr, gf, (*_, M) in zip(ref, fused, basins):
            for m in range(M):
                sr, sf = gr.get_state(m), gf.get_state(m)
                for k in sr:
                    assert np.array_equal(sr[k], sf[k]), (m, k)
            assert list(gf.member_status()) == [0] * M
    finally:
        batch.close()
        for g in ref + fused:
            g.close()


def test_batch_rejects_mixed_code_paths_and_long_calls():
    from mhm_gb300.model import MhmBatch, MhmError, MhmGpu
    basins = _basins()[:2]
    ctxs = _contexts(basins)
    dom, l0, gam, win, M = basins[1]
    other = MhmGpu(dom, proc_soilmoist=2, n_members=M)   # Jarvis stress: the generic code path
    batch = MhmBatch()
    try:
        other.mpr_setup(l0)
        other.mpr(params.random_gammas(M, 2, 0, 1, l0.n_geo, seed=1))
        other.set_meteo(1, *win, on_device=True)
        t0s = [np.ones(b[4], np.int32) for b in basins]
        with pytest.raises(MhmError, match="code paths"):
            batch.run_members([ctxs[0], other], t0s, C)
        with pytest.raises(MhmError):
            batch.run_members(ctxs, t0s, 2 * C)      # more steps than the forcing window holds
    finally:
        batch.close()
        for g in ctxs + [other]:
            g.close()
