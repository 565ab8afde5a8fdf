"""Integer parity of the host-side set-up against the oracle: the routing
order (the library's O(n x sweeps) algorithm vs the reference's literal
O(n^2) sweep, src/mRM/mo_mrm_net_startup.f90:728-886), the network topology
(:630-727) and the per-step calendar (integer Gregorian arithmetic vs the
restated dec2date of newTime - 0.5).  All bit-exact."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from mhm_gb300 import synth

ip = C.POINTER(C.c_int32)


def _p(a):
    return a.ctypes.data_as(ip)


def oracle_order(L, from_n, to_n, n_nodes, n_out):
    perm = np.zeros(n_nodes, np.int32)
    ro = np.zeros(n_nodes, np.int32)
    L.ora_L11_routing_order(n_nodes, n_out, _p(from_n), _p(to_n), _p(perm), _p(ro))
    return perm, ro


def random_forest(rng, n, n_out):
    """A random network of n nodes draining to n_out sinks: every non-sink
    node gets one downstream node among the nodes added before it."""
    order = rng.permutation(n)
    parent = np.full(n, -1)
    for idx in range(n_out, n):
        parent[order[idx]] = order[rng.integers(0, idx)]
    links = [(v + 1, parent[v] + 1) for v in range(n) if parent[v] >= 0]  # in node order, sinks dropped
    from_n = np.full(n, -9999, np.int32)
    to_n = np.full(n, -9999, np.int32)
    for j, (f, t) in enumerate(links):
        from_n[j], to_n[j] = f, t
    return from_n, to_n


@pytest.mark.parametrize("seed", range(6))
def test_routing_order_random_networks(seed, ora_hmath):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 400))
    n_out = int(rng.integers(1, max(2, n // 20)))
    from_n, to_n = random_forest(rng, n, n_out)
    perm, ro = synth.routing_order(from_n, to_n, n, n_out)
    perm_o, ro_o = oracle_order(ora_hmath, from_n, to_n, n, n_out)
    assert np.array_equal(perm, perm_o) and np.array_equal(ro, ro_o)


@pytest.mark.parametrize("kw", [dict(dem_kind="plane"), dict(dem_kind="fractal", ridges=2),
                                dict(dem_kind="fractal", fractal_beta=2.5, tilt=0.0)])
def test_routing_order_synthetic_basins(kw, ora_hmath):
    dom = synth.make_domain(120, 96, 2, 4, seed=7, **kw)
    perm_o, ro_o = oracle_order(ora_hmath, dom.from_n, dom.to_n, dom.n_nodes, dom.n_outlets)
    assert np.array_equal(dom.net_perm, perm_o) and np.array_equal(dom.r_order, ro_o)


@pytest.mark.parametrize("seed", range(6))
def test_oracle_listed_sweep_equals_literal_sweep(seed, ora_hmath):
    """The oracle's listed sweep (used where the literal O(n^2) scan is too
    slow) gives the literal sweep's ranks."""
    from oracle import oracle
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(2, 600))
    n_out = int(rng.integers(1, max(2, n // 20)))
    from_n, to_n = random_forest(rng, n, n_out)
    perm_o, ro_o = oracle_order(ora_hmath, from_n, to_n, n, n_out)
    perm, ro = oracle.routing_order(from_n, to_n, n, n_out, kind="hmath")
    assert np.array_equal(perm, perm_o) and np.array_equal(ro, ro_o)


def test_oracle_listed_sweep_on_the_large_network():
    """62,500 L11 nodes, 1478 levels: the oracle's listed sweep and the
    library's ranks agree (the literal scan does not finish at this size)."""
    from oracle import oracle
    dom = synth.make_domain(1000, 1000, 6, 4, seed=1, dem_kind="fractal", fractal_beta=3.0, tilt=0.0005,
                            ridges=6, order=lambda f, t, n, o: oracle.routing_order(f, t, n, o))
    perm, ro = synth.routing_order(dom.from_n, dom.to_n, dom.n_nodes, dom.n_outlets)
    assert np.array_equal(perm, dom.net_perm) and np.array_equal(ro, dom.r_order)
    assert dom.depth_stats()[0] == 1478


def test_network_topology(ora_hmath):
    dom = synth.make_domain(60, 44, 2, 4, seed=3, dem_kind="fractal", ridges=1)
    L = dom.n_nodes
    fn = np.zeros(L, np.int32)
    tn = np.zeros(L, np.int32)
    id2d = np.ascontiguousarray(dom.id11_2d, np.int32)
    nl = ora_hmath.ora_L11_set_network_topology(dom.nrows11, dom.ncols11, _p(id2d), L, _p(dom.cell_row11),
                                               _p(dom.cell_col11), _p(dom.fdir11), _p(fn), _p(tn))
    assert nl == dom.n_links
    assert np.array_equal(fn, dom.from_n) and np.array_equal(tn, dom.to_n)


@pytest.mark.parametrize("jul_start,timestep,n", [(synth.JUL_2000, 1, 24 * 800), (2415021, 1, 24 * 400),
                                                 (2451545 + 59, 3, 8 * 1500), (2440588, 6, 4 * 2000),
                                                 (2459000, 24, 3000), (2458849, 2, 12 * 370)])
def test_step_calendar(jul_start, timestep, n, lib, ora_hmath):
    m, h, d = (np.zeros(n, np.int32) for _ in range(3))
    assert lib.mhm_step_calendar(jul_start, timestep, 1, n, _p(m), _p(h), _p(d)) == 0
    mo, ho, do = (np.zeros(n, np.int32) for _ in range(3))
    ora_hmath.ora_step_calendar(jul_start, timestep, n, _p(mo), _p(ho), _p(do), None, None)
    assert np.array_equal(m, mo) and np.array_equal(h, ho) and np.array_equal(d, do)


def _topology(lib, nrows, ncols, id2d, rows, cols, fdir):
    n = len(fdir)
    fn = np.zeros(n, np.int32)
    tn = np.zeros(n, np.int32)
    nl = np.zeros(1, np.int32)
    rc = lib.mhm_network_topology(nrows, ncols, _p(np.ascontiguousarray(id2d, np.int32)), n,
                                  _p(np.ascontiguousarray(rows, np.int32)), _p(np.ascontiguousarray(cols, np.int32)),
                                  _p(np.ascontiguousarray(fdir, np.int32)), _p(fn), _p(tn), _p(nl))
    assert rc == 0
    return fn, tn, int(nl[0])


def test_native_network_topology_matches_oracle(lib, ora_hmath):
    dom = synth.make_domain(60, 44, 2, 4, seed=3, dem_kind="fractal", ridges=1)
    fn, tn, nl = _topology(lib, dom.nrows11, dom.ncols11, dom.id11_2d, dom.cell_row11, dom.cell_col11, dom.fdir11)
    assert nl == dom.n_links
    assert np.array_equal(fn, dom.from_n) and np.array_equal(tn, dom.to_n)


def test_native_network_topology_reproduces_case00(lib):
    """check/case_00's L11 flow directions give exactly the L11_fromN / L11_toN
    its mRM restart file holds (integer parity of the network set-up)."""
    z = np.load(Path(__file__).resolve().parent / "golden" / "case00_run.npz")
    mask = z["mask11"].astype(bool)                 # [ncols][nrows]
    ncols, nrows = mask.shape
    jj, ii = np.nonzero(mask)                       # packing order (row index fastest)
    n = int(mask.sum())
    id2d = np.full(mask.shape, -9999, np.int32)
    id2d[mask] = np.arange(1, n + 1)
    fn, tn, nl = _topology(lib, nrows, ncols, id2d, ii + 1, jj + 1, z["l11_fdir"])
    assert nl == n - 1
    assert np.array_equal(fn, z["from_n"]) and np.array_equal(tn, z["to_n"])
    # and the routing order built from them is the reference's netPerm / rOrder
    perm = np.zeros(n, np.int32)
    ro = np.zeros(n, np.int32)
    assert lib.mhm_routing_order(n, 1, _p(fn), _p(tn), _p(perm), _p(ro)) == 0
    assert np.array_equal(perm, z["net_perm"]) and np.array_equal(ro, z["r_order"])
