"""Serving loop: continuous batching of mHM + mRM runs on one GPU.

A request is one forecast run on a basin of the catalogue: a global
parameter vector (regionalised on the device by MPR), a horizon in hourly
steps and a warm start from the basin's restart state, which stays resident
on the device as a snapshot.  The server keeps, per basin with work, one
context whose members are request slots; the loop

  1. admits waiting requests into free slots of idle contexts (device MPR
     for the slot, the restart snapshot loaded into it) -- creating a basin's
     context only when its device footprint fits the HBM budget, and
     retiring contexts that have gone idle to make room;
  2. enqueues one chunk of steps on every idle context with work, each
     member at its own model step (mhm_run_members_async), so the contexts'
     kernels overlap on the device;
  3. polls the contexts without waiting (mhm_poll) and, for each whose chunk
     has completed, hands its active slots their chunk of outlet discharge,
     frees the slots whose horizon is complete and makes the context idle --
     every context advances at its own pace.

Requests that arrive while others run join at the next chunk boundary of
their basin's context.  A member's arithmetic does not depend on the other
members, the slot it occupies or when it was admitted, so each result equals
the same run executed alone (`run_alone`).

Forcing: each basin has a device-resident window of `chunk` hourly rows that
every chunk of every run reads (the synthetic forecast repeats every
`chunk` steps), so admitting a run at any chunk boundary reads the same
forcing it would alone.

Failures stay with the request that caused them (the reference's only
error path is error_message -> stop of the whole program,
src/MPR/mo_multi_param_reg.f90:314,422):
  * a request whose parameter vector has the wrong length or non-finite
    entries, or whose basin alone exceeds the HBM budget, is rejected at
    submission;
  * a regionalisation that fails (MhmError) fails that request only;
  * a member whose states or discharge turn non-finite during a chunk
    (mhm_member_status) is failed and its slot freed at the chunk boundary;
  * a request can be cancelled at any time; it leaves at the next chunk
    boundary of its context;
  * a request's `on_chunk` consumer (e.g. streaming each chunk's discharge
    to a client) runs on a worker thread; if it raises, that request is
    failed and its slot freed at the next boundary.
The other requests continue and finish with the results they give alone.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from concurrent.futures import Future, ThreadPoolExecutor

from . import params as gparams
from . import synth
from .model import MhmError, MhmGpu


@dataclass
class Basin:
    name: str
    dom: synth.Domain
    l0: synth.L0Maps
    window: tuple = ()          # device forcing window (pre, temp, pet) [chunk, N]
    restart: dict | None = None  # host copy of the spun-up state (for run_alone)

    @property
    def n_cells(self) -> int:
        return self.dom.n_cells


@dataclass
class Request:
    rid: int
    basin: int
    gamma: np.ndarray
    horizon: int                 # hourly steps
    arrival: float = 0.0         # seconds after the start of the run
    admitted: float | None = None
    done: float | None = None
    q: list = field(default_factory=list)
    status: str = "pending"      # pending, running, done, failed, rejected, cancelled
    error: str | None = None
    on_chunk: object = None      # optional consumer f(request, discharge chunk [gauge, step])
    cancelled: bool = False
    futures: list = field(default_factory=list)

    def discharge(self) -> np.ndarray:
        """Outlet discharge [gauge, step] over the horizon."""
        return np.concatenate(self.q, axis=1)[:, :self.horizon]

    @property
    def latency(self) -> float:
        return (self.done - self.arrival) if self.done is not None else math.nan


def context_bytes(basin: Basin, members: int, chunk: int, chunk_bytes: float = 8e9) -> int:
    """Device footprint of a context with `members` slots (the library's
    allocations: parameters, states, two runoff chunk slots, routing chunk
    series, restart snapshot, forcing window, MPR tables)."""
    N, H, L = basin.dom.n_cells, basin.dom.n_horizons, basin.dom.n_nodes
    planes = 16 + 24 + 5 * H
    tc = max(1, min(chunk, int(chunk_bytes // (2 * members * N * 8))))
    b = members * (planes + 5 + H) * N * 8                # parameters + states
    b += 2 * tc * members * N * 8                          # runoff chunk slots
    b += 3 * members * tc * L * 8 + 8 * members * L * 8    # routing series + states + C1/C2
    b += ((5 + H) * N + 4 * L) * 8                         # restart snapshot
    b += 3 * chunk * N * 8                                 # forcing window
    b += basin.l0.n_cells0 * 24 + members * 64 * 1024      # L0 slots, MPR tables
    return int(b)


class Server:
    """Continuous-batching request loop over a catalogue of basins."""

    def __init__(self, basins: list[Basin], hbm_budget: float = 150e9, chunk: int = 240, max_slots: int = 16,
                 proc_sm: int = 1, proc_pet: int = 0, spinup_steps: int = 90 * 24, gamma_spinup=None,
                 autotune: bool = False, backend=MhmGpu, window_fn=None, workers: int = 4, fused: bool = False):
        """`backend` builds a basin's context (MhmGpu); `window_fn(basin)`
        gives its forcing window (default: the synthetic forecast window in
        device memory).  `fused`: the chunks enqueued in one pass of the loop
        run their cell chains in one persistent launch (MhmBatch) -- every
        context whose chunk fits one launch chunk; the others run alone."""
        self.backend = backend
        self.batch = None
        if fused and backend is MhmGpu:
            from .model import MhmBatch
            self.batch = MhmBatch()
        self.basins = basins
        self.budget = hbm_budget
        self.chunk = chunk
        self.max_slots = max_slots
        self.proc_sm, self.proc_pet = proc_sm, proc_pet
        self.ctx: dict[int, dict] = {}          # basin -> {g, slots, tt0, bytes}
        self.used = 0
        self.waiting: list[Request] = []
        self.finished: list[Request] = []
        self.iterations = 0
        self.cell_steps = 0
        self.autotune = autotune
        self.tuned: dict[str, dict] = {}
        self.failed: list[Request] = []      # failed, rejected or cancelled
        # admission statistics: contexts opened and retired to make room,
        # admissions deferred by the HBM budget, peak device footprint and
        # peak number of running requests
        self.stats = {"contexts_opened": 0, "contexts_retired_for_room": 0, "budget_deferrals": 0,
                      "peak_hbm_bytes": 0, "peak_running": 0}
        self._cancel: set[int] = set()       # request ids to cancel (filled from any thread)
        self.pool = ThreadPoolExecutor(max_workers=workers)
        for b in basins:
            if not b.window:
                b.window = window_fn(b) if window_fn else device_window(b.dom, chunk)
            if b.restart is None:
                b.restart = self._spin_up(b, spinup_steps, gamma_spinup)

    # ---- basin set-up ----
    def _spin_up(self, b: Basin, steps: int, gamma) -> dict:
        """Default states advanced `steps` hourly steps with the namelist
        parameters: the warm start every request of the basin begins from."""
        g = self.backend(b.dom, proc_soilmoist=self.proc_sm, proc_pet=self.proc_pet, n_members=1)
        try:
            g.mpr_setup(b.l0)
            gam = gamma if gamma is not None else gparams.default_gamma(self.proc_sm, self.proc_pet, 1, b.l0.n_geo)
            g.mpr(gam)
            g.init_states(0)
            for c in range(math.ceil(steps / self.chunk)):   # steps == 0: default states
                n = min(self.chunk, steps - c * self.chunk)
                tt0 = 1 + c * self.chunk
                g.set_meteo(tt0, *[w[:n] for w in b.window], on_device=True)
                g.run(tt0, n)
            # states only: the Muskingum coefficients of a run come from its
            # own parameter vector (mhm_mpr), not from the spin-up
            return {k: v for k, v in g.get_state(0).items() if k not in ("C1", "C2")}
        finally:
            g.close()

    def _open(self, bi: int, members: int) -> bool:
        b = self.basins[bi]
        need = context_bytes(b, members, self.chunk)
        if self.used + need > self.budget:
            return False
        g = self.backend(b.dom, proc_soilmoist=self.proc_sm, proc_pet=self.proc_pet, n_members=members,
                         read_states=True)
        g.mpr_setup(b.l0)
        g.snapshot_alloc(1)
        g.set_state(b.restart, 0)
        g.snapshot_save(0, 0)
        g.set_meteo(1, *b.window, on_device=True)
        if self.autotune:
            # time the variants on the basin's first chunk with the namelist
            # parameters and the warm start in every slot (states restored after)
            g.mpr(np.tile(gparams.default_gamma(self.proc_sm, self.proc_pet, 1, b.l0.n_geo), (members, 1)))
            for m in range(members):
                g.snapshot_load(0, m)
            t = g.autotune(1, self.chunk)
            self.tuned[b.name] = {k: t[k] for k in ("cell_blocks_per_sm", "route_sub_steps")}
        self.ctx[bi] = {"g": g, "bi": bi, "slots": [None] * members, "tt0": np.zeros(members, np.int32), "bytes": need,
                        "q": np.zeros((members, len(b.dom.gauge_node), self.chunk)), "busy": False}
        self.used += need
        self.stats["contexts_opened"] += 1
        self.stats["peak_hbm_bytes"] = max(self.stats["peak_hbm_bytes"], self.used)
        return True

    def _close(self, bi: int):
        c = self.ctx.pop(bi)
        c["g"].close()
        self.used -= c["bytes"]

    # ---- the loop ----
    def _fail(self, r: Request, status: str, error: str | None):
        r.status, r.error = status, error
        r.done = (time.perf_counter() - self._t0) if hasattr(self, "_t0") else 0.0
        self.failed.append(r)

    def submit(self, r: Request):
        """Queue a request; malformed ones are rejected here."""
        b = self.basins[r.basin] if 0 <= r.basin < len(self.basins) else None
        if b is None:
            return self._fail(r, "rejected", "unknown basin")
        n_gamma = int(gparams.offsets(self.proc_sm, self.proc_pet, 1, b.l0.n_geo)[10])
        g = np.asarray(r.gamma, np.float64)
        if g.shape != (n_gamma,):
            return self._fail(r, "rejected", f"parameter vector has shape {g.shape}, expected ({n_gamma},)")
        if not np.all(np.isfinite(g)):
            return self._fail(r, "rejected", "parameter vector has non-finite entries")
        if r.horizon < 1:
            return self._fail(r, "rejected", "horizon must be at least one step")
        if context_bytes(b, 1, self.chunk) > self.budget:
            return self._fail(r, "rejected", "the basin alone exceeds the HBM budget")
        self.waiting.append(r)

    def cancel(self, rid: int):
        """Cancel a request (callable from any thread, e.g. a consumer): the
        loop drops a waiting request at its next pass and a running one at
        its context's next chunk boundary."""
        self._cancel.add(rid)

    def _apply_cancels(self):
        if not self._cancel:
            return
        rids = set(self._cancel)
        self._cancel -= rids
        still = []
        for r in self.waiting:
            if r.rid in rids:
                r.cancelled = True
                self._fail(r, "cancelled", None)
            else:
                still.append(r)
        self.waiting = still
        for c in self.ctx.values():
            for r in c["slots"]:
                if r is not None and r.rid in rids:
                    r.cancelled = True

    def _release(self, c: dict, m: int):
        """Free slot m of a context whose chunk is not in flight."""
        r = c["slots"][m]
        c["slots"][m] = None
        c["tt0"][m] = 0
        return r

    def _sweep(self, c: dict):
        """At a chunk boundary: slots of cancelled requests and of requests
        whose consumer raised are freed."""
        for m, r in enumerate(c["slots"]):
            if r is None:
                continue
            err = next((f.exception() for f in r.futures if f.done() and f.exception() is not None), None)
            if r.cancelled:
                self._release(c, m)
                self._fail(r, "cancelled", None)
            elif err is not None:
                self._release(c, m)
                self._fail(r, "failed", f"chunk consumer raised {type(err).__name__}: {err}")

    def _admit(self, now: float):
        still = []
        for r in self.waiting:
            if r.arrival > now:
                still.append(r)
                continue
            c = self.ctx.get(r.basin)
            if c is not None and c["busy"]:
                still.append(r)          # its chunk in flight: admit at the next completion
                continue
            if c is None:
                want = min(self.max_slots, max(1, sum(1 for w in self.waiting
                                                      if w.basin == r.basin and w.arrival <= now)))
                if not self._open(r.basin, want):
                    # make room: retire contexts without active slots
                    for bi in [k for k, v in self.ctx.items() if all(s is None for s in v["slots"])]:
                        self._close(bi)
                        self.stats["contexts_retired_for_room"] += 1
                    if not self._open(r.basin, want):
                        self.stats["budget_deferrals"] += 1
                        still.append(r)
                        continue
                c = self.ctx[r.basin]
            try:
                slot = c["slots"].index(None)
            except ValueError:
                still.append(r)
                continue
            g = c["g"]
            try:
                g.mpr(r.gamma, member0=slot)
            except MhmError as e:          # this request only
                self._fail(r, "failed", f"regionalisation failed: {e}")
                continue
            g.snapshot_load(0, slot)
            c["slots"][slot] = r
            c["tt0"][slot] = 1
            r.admitted = now
            r.status = "running"
        self.waiting = still
        running = sum(1 for c in self.ctx.values() for sl in c["slots"] if sl is not None)
        self.stats["peak_running"] = max(self.stats["peak_running"], running)

    def step(self, now: float) -> bool:
        """One pass of the loop; returns False when there is nothing to do.
        Every context advances at its own pace: a chunk is enqueued on each
        idle context with active slots, and a context whose chunk has
        completed (mhm_poll, no waiting) is finished and can take its next
        chunk and new requests at once -- a small basin is not held back by
        the chunk of a large one."""
        self._apply_cancels()
        for c in self.ctx.values():
            if not c["busy"]:
                self._sweep(c)
        self._admit(now)
        ready = [c for c in self.ctx.values() if not c["busy"] and any(s is not None for s in c["slots"])]
        together = []
        for c in ready:
            tt0 = np.where([s is not None for s in c["slots"]], c["tt0"], 0).astype(np.int32)
            c["tt0_now"] = tt0
            # one launch chunk covers the call when its two runoff slots fit the library's budget
            fits = 2 * len(c["slots"]) * self.basins[c["bi"]].n_cells * 8 * self.chunk <= 8 * 2 ** 30
            if self.batch is not None and fits:
                together.append(c)
            else:
                c["g"].run_members_async(tt0, self.chunk, c["q"])
            c["busy"] = True
        if together:
            self.batch.run_members([c["g"] for c in together], [c["tt0_now"] for c in together], self.chunk,
                                   [c["q"] for c in together])
        busy = [(bi, c) for bi, c in self.ctx.items() if c["busy"]]
        if not busy:
            return False
        progressed = False
        for bi, c in busy:
            if not c["g"].poll():
                continue
            c["g"].sync()                          # host side of the chunk (gauge series)
            status = c["g"].member_status()        # non-finite members of this chunk
            c["busy"] = False
            progressed = True
            t_done = time.perf_counter()
            n = self.basins[bi].n_cells
            for m, r in enumerate(c["slots"]):
                if r is None or c["tt0_now"][m] <= 0:
                    continue
                if status[m] != 0:
                    self._release(c, m)
                    self._fail(r, "failed", "non-finite states or discharge")
                    continue
                chunk_q = c["q"][m].copy()
                r.q.append(chunk_q)
                if r.on_chunk is not None:
                    r.futures.append(self.pool.submit(r.on_chunk, r, chunk_q))
                self.cell_steps += n * self.chunk
                c["tt0"][m] += self.chunk
                if c["tt0"][m] - 1 >= r.horizon:
                    r.done = t_done - self._t0
                    r.status = "done"
                    self.finished.append(r)
                    c["slots"][m] = None
        if not progressed:
            time.sleep(2e-4)
        self.iterations += 1
        return True

    def serve(self, requests: list[Request], timeout_s: float = 600.0) -> dict:
        """Run until every request is finished; arrivals follow their
        `arrival` offsets in wall-clock time."""
        self._t0 = time.perf_counter()
        for r in requests:
            self.submit(r)
        while (self.waiting or any(any(s is not None for s in c["slots"]) for c in self.ctx.values())):
            now = time.perf_counter() - self._t0
            if now > timeout_s:
                raise TimeoutError("serving loop did not drain in time")
            if not self.step(now):
                nxt = min((r.arrival for r in self.waiting), default=now)
                time.sleep(max(0.0, min(0.05, nxt - now)))
        wall = time.perf_counter() - self._t0
        for bi in list(self.ctx):
            self._close(bi)
        # a consumer that raised on a request's last chunk fails it too
        for r in list(self.finished):
            err = next((f.exception() for f in r.futures if f.exception() is not None), None)
            if err is not None:
                self.finished.remove(r)
                r.status, r.error = "failed", f"chunk consumer raised {type(err).__name__}: {err}"
                self.failed.append(r)
        out = summarize(self.finished, wall, self.cell_steps)
        out["failed"] = len(self.failed)
        waits = np.array([r.admitted - r.arrival for r in self.finished if r.admitted is not None])
        out["admission"] = dict(self.stats, queue_wait_p50_s=float(np.percentile(waits, 50)) if waits.size else None,
                                queue_wait_p99_s=float(np.percentile(waits, 99)) if waits.size else None,
                                rejected=sum(1 for r in self.failed if r.status == "rejected"),
                                cancelled=sum(1 for r in self.failed if r.status == "cancelled"))
        return out

    def close(self):
        for bi in list(self.ctx):
            self._close(bi)
        self.pool.shutdown(wait=True)
        if self.batch is not None:
            self.batch.close()
            self.batch = None


def device_window(dom, chunk: int) -> tuple:
    """The synthetic forecast window of a basin in device memory."""
    import torch
    f = synth.make_forcing(dom, chunk, seed=2)
    return tuple(torch.from_numpy(f[k]).cuda() for k in ("pre", "temp", "pet"))


def summarize(done: list[Request], wall: float, cell_steps: int) -> dict:
    lat = np.array([r.latency for r in done])
    return {"requests": len(done), "wall_s": wall, "throughput": cell_steps / wall,
            "p50_s": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_s": float(np.percentile(lat, 99)) if lat.size else None}


def run_alone(basin: Basin, r: Request, chunk: int, proc_sm: int = 1, proc_pet: int = 0,
              g: MhmGpu | None = None) -> np.ndarray:
    """The request on its own: one-member context, the ordinary mhm_run path,
    same warm start and forcing window.  Returns [gauge, step]."""
    own = g is None
    if own:
        g = MhmGpu(basin.dom, proc_soilmoist=proc_sm, proc_pet=proc_pet, n_members=1, read_states=True)
        g.mpr_setup(basin.l0)
    try:
        g.mpr(r.gamma)
        g.set_state(basin.restart, 0)
        qs = []
        for c in range(math.ceil(r.horizon / chunk)):
            tt0 = 1 + c * chunk
            g.set_meteo(tt0, *basin.window, on_device=True)
            qs.append(g.run(tt0, chunk)[0])
        return np.concatenate(qs, axis=1)[:, :r.horizon]
    finally:
        if own:
            g.close()


def serve_plain(basins: list[Basin], requests: list[Request], chunk: int, proc_sm: int = 1,
                proc_pet: int = 0) -> dict:
    """The one-run-at-a-time path: requests in arrival order, each on a
    one-member context of its basin (contexts kept per basin)."""
    ctxs: dict[int, MhmGpu] = {}
    t0 = time.perf_counter()
    cell_steps = 0
    try:
        for r in sorted(requests, key=lambda q: q.arrival):
            now = time.perf_counter() - t0
            if r.arrival > now:
                time.sleep(r.arrival - now)
            b = basins[r.basin]
            if r.basin not in ctxs:
                g = MhmGpu(b.dom, proc_soilmoist=proc_sm, proc_pet=proc_pet, n_members=1, read_states=True)
                g.mpr_setup(b.l0)
                ctxs[r.basin] = g
            r.q = [run_alone(b, r, chunk, proc_sm, proc_pet, g=ctxs[r.basin])]
            r.done = time.perf_counter() - t0
            cell_steps += b.n_cells * chunk * math.ceil(r.horizon / chunk)
        wall = time.perf_counter() - t0
    finally:
        for g in ctxs.values():
            g.close()
    return summarize(requests, wall, cell_steps)


def run_batched(basins: list[Basin], requests: list[Request], chunk: int, proc_sm: int = 1,
                proc_pet: int = 0) -> dict:
    """Many whole runs at once (the uneven-basins workload): one context per
    request, all advanced in rounds of one chunk; each round is ONE
    persistent cell-chain launch over every run still active (MhmBatch, a
    device work queue of tiles), then each run's accumulation and routing on
    its own streams.  Rounds are enqueued without waiting: the library keeps
    two chunks per context in flight (the cell chain of round k overlaps the
    routing of round k-1).  Context set-up (MPR, warm start) is inside the
    timed region, as in serve_plain.  Results equal run_alone's."""
    from .model import MhmBatch
    t0 = time.perf_counter()
    ctxs: dict[int, MhmGpu] = {}
    batch = MhmBatch()
    cell_steps = 0
    try:
        for r in requests:
            b = basins[r.basin]
            g = MhmGpu(b.dom, proc_soilmoist=proc_sm, proc_pet=proc_pet, n_members=1, read_states=True)
            g.mpr_setup(b.l0)
            g.mpr(r.gamma)
            g.set_state(b.restart, 0)
            g.set_meteo(1, *b.window, on_device=True)
            ctxs[r.rid] = g
            r.q = []
        rounds = max(math.ceil(r.horizon / chunk) for r in requests)
        for k in range(rounds):
            active = [r for r in requests if k * chunk < r.horizon]
            qs = [np.zeros((1, len(basins[r.basin].dom.gauge_node), chunk)) for r in active]
            batch.run_members([ctxs[r.rid] for r in active], [np.array([1 + k * chunk], np.int32)] * len(active),
                              chunk, qs)
            for r, q in zip(active, qs):
                r.q.append(q[0])
                cell_steps += basins[r.basin].n_cells * chunk
        for r in requests:
            ctxs[r.rid].sync()
            r.done = time.perf_counter() - t0
            r.status = "done"
        wall = time.perf_counter() - t0
    finally:
        batch.close()
        for g in ctxs.values():
            g.close()
    return summarize(requests, wall, cell_steps)


def make_catalogue(n: int, seed: int = 11, n_min: float = 1e3, n_max: float = 1e6, l0_factor: int = 2,
                   h_min: int = 2, h_max: int = 6, include_max: bool = False) -> list[Basin]:
    """Basins with cell counts log-uniform in [n_min, n_max] (square-ish L1
    grids), h_min..h_max soil horizons, their own fractal DEM / D8 network;
    with include_max the last basin has n_max cells."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        cells = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        if include_max and i == n - 1:
            cells = n_max
        nr = max(8, int(round(math.sqrt(cells))))
        nc = max(8, int(round(cells / nr)))
        H = int(rng.integers(h_min, h_max + 1))
        dom = synth.make_domain(nr, nc, H, l11_factor=4 if nr * nc > 4e4 else 2, seed=100 + i, dem_kind="fractal",
                                fractal_beta=3.0, tilt=0.001)
        l0 = synth.make_l0(dom, l0_factor, seed=200 + i)
        out.append(Basin(name=f"basin{i}_{nr}x{nc}_H{H}", dom=dom, l0=l0))
    return out


def make_requests(basins: list[Basin], n: int, rate: float, seed: int = 12, h_min_days: int = 30,
                  h_max_days: int = 365, proc_sm: int = 1, proc_pet: int = 0) -> list[Request]:
    """Poisson arrivals at `rate` per second; each request a basin of the
    catalogue, a parameter vector within the namelist bounds and a horizon
    of h_min..h_max days hourly."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = []
    for i in range(n):
        bi = int(rng.integers(0, len(basins)))
        g = gparams.random_gammas(1, proc_sm, proc_pet, 1, basins[bi].l0.n_geo, seed=int(rng.integers(1 << 30)))[0]
        days = int(rng.integers(h_min_days, h_max_days + 1))
        reqs.append(Request(rid=i, basin=bi, gamma=g, horizon=24 * days, arrival=float(t[i])))
    return reqs
