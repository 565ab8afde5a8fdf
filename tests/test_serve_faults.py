"""Failure isolation in the serving loop, on the CPU: the request loop of
mhm_gb300.serve driven by a stand-in context that computes a simple
per-member recurrence on the host (so the host-side logic -- admission,
chunk boundaries, member status, cancellation, consumer threads -- runs
without a GPU).  Every kind of fault must fail its own request only; the
others finish with exactly the discharge they give when run alone."""
import numpy as np

from mhm_gb300 import params, serve, synth
from mhm_gb300.model import MhmError

CHUNK = 24


class FakeCtx:
    """Stand-in for MhmGpu: member m carries a storage s; each step
    s <- 0.9 s + 1e-3 sum(gamma_m) and the outlet discharge is s.  A
    parameter set with gamma[0] > 1e3 makes the storage NaN (a member whose
    states turn non-finite); gamma[1] == -999 makes the regionalisation
    fail."""

    def __init__(self, dom, proc_soilmoist=1, proc_pet=0, n_members=1, read_states=False, **_):
        self.M = n_members
        self.G = len(dom.gauge_node)
        self.s = np.zeros(n_members)
        self.k = np.zeros(n_members)
        self.snap = {}
        self.flags = np.zeros(n_members, np.int32)
        self.closed = False

    def mpr_setup(self, l0):
        pass

    def mpr(self, gammas, member0=0):
        g = np.atleast_2d(gammas)
        for i, row in enumerate(g):
            if row[1] == -999.0:
                raise MhmError("mhm_mpr failed (-1): bad parameter vector")
            self.k[member0 + i] = np.nan if row[0] > 1e3 else 1e-3 * float(np.sum(row))

    def init_states(self, m=0):
        self.s[m] = 1.0

    def set_meteo(self, *a, **k):
        pass

    def _advance(self, m, n):
        out = np.zeros(n)
        for t in range(n):
            self.s[m] = 0.9 * self.s[m] + self.k[m]
            out[t] = self.s[m]
        if not np.isfinite(self.s[m]):
            self.flags[m] = 1
        return out

    def run(self, tt0, n):
        q = np.zeros((self.M, self.G, n))
        for m in range(self.M):
            q[m, :, :] = self._advance(m, n)
        return q

    def get_state(self, m=0):
        return {"s": np.array([self.s[m]])}

    def set_state(self, st, m=0):
        self.s[m] = float(st["s"][0])

    def snapshot_alloc(self, n):
        pass

    def snapshot_save(self, m, slot):
        self.snap[slot] = self.s[m]

    def snapshot_load(self, slot, m):
        self.s[m] = self.snap[slot]

    def autotune(self, tt0, n):
        return {"cell_blocks_per_sm": 4, "route_sub_steps": 8}

    def run_members_async(self, tt0, n, q):
        for m in range(self.M):
            q[m] = 0.0
            if tt0[m] > 0:
                q[m, :, :] = self._advance(m, n)

    def poll(self):
        return True

    def sync(self):
        pass

    def member_status(self):
        st = np.where(self.flags != 0, -5, 0).astype(np.int32)
        self.flags[:] = 0
        return st

    def close(self):
        self.closed = True


def _basins():
    out = []
    for i, (nr, nc) in enumerate([(8, 8), (12, 10)]):
        dom = synth.make_domain(nr, nc, 2, l11_factor=2, seed=100 + i)
        l0 = synth.make_l0(dom, 2, seed=200 + i)
        out.append(serve.Basin(name=f"b{i}", dom=dom, l0=l0))
    return out


def _server(basins, budget=150e9):
    return serve.Server(basins, hbm_budget=budget, chunk=CHUNK, max_slots=4, spinup_steps=2 * CHUNK,
                        backend=FakeCtx, window_fn=lambda b: ("window",))


def test_every_fault_fails_only_its_own_request():
    basins = _basins()
    srv = _server(basins)
    n_geo = basins[0].l0.n_geo
    good = params.random_gammas(4, 1, 0, 1, n_geo, seed=5)
    reqs = [serve.Request(rid=i, basin=i % 2, gamma=good[i], horizon=3 * CHUNK) for i in range(4)]
    bad = []
    g = good[0].copy()
    bad.append(serve.Request(rid=10, basin=0, gamma=g[:-1], horizon=CHUNK))            # wrong length
    g = good[1].copy()
    g[3] = np.nan
    bad.append(serve.Request(rid=11, basin=1, gamma=g, horizon=CHUNK))                 # non-finite entry
    g = good[2].copy()
    g[0] = 1e6
    bad.append(serve.Request(rid=12, basin=0, gamma=g, horizon=3 * CHUNK))             # NaN states on device
    g = good[3].copy()
    g[1] = -999.0
    bad.append(serve.Request(rid=13, basin=1, gamma=g, horizon=CHUNK))                 # regionalisation fails

    def boom(r, q):
        raise RuntimeError("client went away")

    bad.append(serve.Request(rid=14, basin=0, gamma=good[1], horizon=3 * CHUNK, on_chunk=boom))
    streamed = []
    reqs[1].on_chunk = lambda r, q: streamed.append(q.shape)

    def cancel_me(r, q):
        srv.cancel(r.rid)

    bad.append(serve.Request(rid=15, basin=1, gamma=good[2], horizon=5 * CHUNK, on_chunk=cancel_me))
    try:
        res = srv.serve(reqs + bad, timeout_s=60)
    finally:
        srv.close()
    assert res["requests"] == 4 and res["failed"] == 6
    status = {r.rid: (r.status, r.error) for r in reqs + bad}
    assert status[10][0] == "rejected" and "shape" in status[10][1]
    assert status[11][0] == "rejected" and "non-finite" in status[11][1]
    assert status[12] == ("failed", "non-finite states or discharge")
    assert status[13][0] == "failed" and "regionalisation" in status[13][1]
    assert status[14][0] == "failed" and "client went away" in status[14][1]
    assert status[15][0] == "cancelled"
    assert len(streamed) == 3
    for r in reqs:
        assert r.status == "done"
        alone = serve.run_alone(basins[r.basin], r, CHUNK, g=FakeCtx(basins[r.basin].dom))
        assert np.array_equal(r.discharge(), alone)


def test_over_budget_basin_is_rejected_and_others_run():
    basins = _basins()
    small_budget = serve.context_bytes(basins[0], 1, CHUNK) * 1.5   # basin 1 alone does not fit
    assert serve.context_bytes(basins[1], 1, CHUNK) > small_budget
    srv = _server(basins, budget=small_budget)
    gam = params.random_gammas(2, 1, 0, 1, basins[0].l0.n_geo, seed=6)
    reqs = [serve.Request(rid=0, basin=0, gamma=gam[0], horizon=2 * CHUNK),
            serve.Request(rid=1, basin=1, gamma=gam[1], horizon=2 * CHUNK)]
    try:
        res = srv.serve(reqs, timeout_s=60)
    finally:
        srv.close()
    assert reqs[0].status == "done" and res["requests"] == 1
    assert reqs[1].status == "rejected" and "budget" in reqs[1].error
    adm = res["admission"]
    assert adm["rejected"] == 1 and adm["contexts_opened"] == 1 and adm["peak_running"] == 1
    assert 0 < adm["peak_hbm_bytes"] <= small_budget and adm["queue_wait_p50_s"] >= 0.0


def test_budget_defers_admission_until_a_context_retires():
    """Two basins that fit the budget only one at a time: the second request
    waits (a budget deferral) until the first basin's context is idle and is
    retired to make room, then runs; both give their stand-alone results."""
    basins = _basins()
    b0, b1 = (serve.context_bytes(basins[i], 1, CHUNK) for i in (0, 1))
    srv = _server(basins, budget=max(b0, b1) * 1.01)
    gam = params.random_gammas(2, 1, 0, 1, basins[0].l0.n_geo, seed=8)
    reqs = [serve.Request(rid=0, basin=0, gamma=gam[0], horizon=2 * CHUNK),
            serve.Request(rid=1, basin=1, gamma=gam[1], horizon=CHUNK)]
    try:
        res = srv.serve(reqs, timeout_s=60)
    finally:
        srv.close()
    assert [r.status for r in reqs] == ["done", "done"]
    adm = res["admission"]
    assert adm["budget_deferrals"] >= 1 and adm["contexts_retired_for_room"] >= 1
    assert adm["contexts_opened"] == 2 and adm["peak_hbm_bytes"] <= max(b0, b1) * 1.01
    for r in reqs:
        alone = serve.run_alone(basins[r.basin], r, CHUNK, g=FakeCtx(basins[r.basin].dom))
        assert np.array_equal(r.discharge(), alone)


def test_cancel_while_waiting():
    basins = _basins()
    srv = _server(basins)
    gam = params.random_gammas(1, 1, 0, 1, basins[0].l0.n_geo, seed=7)[0]
    r = serve.Request(rid=3, basin=0, gamma=gam, horizon=CHUNK, arrival=30.0)
    srv._t0 = 0.0
    srv.submit(r)
    srv.cancel(3)
    srv.step(now=0.0)
    assert r.status == "cancelled" and not srv.waiting
    srv.close()
