"""Scenarios the bounds-checked build is run on (tests/test_gpu_bounds_check.py):
each returns its discharge and states, so that the bounds-checked library's
results can be compared with the default library's.  Run as a script with
MHM_BOUNDS_CHECK=1 it writes them, the library's build flag, the device
status after every scenario and the self-test's report to an npz file."""
import os
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

from mhm_gb300 import params, synth  # noqa: E402


def _flat(st):
    return np.concatenate([np.asarray(v, np.float64).reshape(-1) for _, v in sorted(st.items())])


def ensemble_chunks(status):
    """8 members (member-tiled blocks), device MPR, chunked calls, cluster-walk routing"""
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(30, 26, 3, l11_factor=2, seed=21, dem_kind="fractal", ridges=1)
    l0 = synth.make_l0(dom, 2, seed=22)
    gam = params.random_gammas(8, 1, 0, 1, l0.n_geo, seed=23)
    f = synth.make_forcing(dom, 96, seed=24)
    g = MhmGpu(dom, n_members=8)
    try:
        g.set_launch_config(cell_blocks_per_sm=8, route_sub_steps=4, chunk_steps=40, route_cluster=8)
        g.mpr_setup(l0)
        g.mpr(gam)
        for m in range(8):
            g.init_states(m)
        g.set_meteo(1, **f)
        q = np.concatenate([g.run(1, 50), g.run(51, 46)], axis=2)
        status.append(g.device_status())
        return q.reshape(-1), _flat(g.get_state(7))
    finally:
        g.close()


def inflow_window(status):
    """inflow gauges (a headwater and a cutting one), adaptive routing windows"""
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(12, 10, 3, l11_factor=4, seed=1, cellsize_m=3000.0)
    p = synth.make_eff_params(dom, seed=3)
    f = synth.make_forcing(dom, 96, seed=2, gamma_theta=4.0)
    nl = dom.n_links
    up = np.bincount(dom.to_n[:nl] - 1, minlength=dom.n_nodes)
    outlet = int(dom.gauge_node[0]) - 1
    order = [v for v in np.argsort(-up, kind="stable") if v != outlet and up[v] > 0]
    node = np.array([order[0] + 1, order[1] + 1], np.int32)
    q_in = np.random.default_rng(9).uniform(0.5, 20.0, (6, 2))
    g = MhmGpu(dom, proc_routing=2)
    try:
        g.prepare(p, np.array([1.5, 0, 0, 0, 0]))
        g.set_inflow_gauges(node, np.array([0, 1], np.int32), q_in, day0=1)
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        q = np.concatenate([g.run(1, 48), g.run(49, 48)], axis=2)
        status.append(g.device_status())
        return q.reshape(-1), _flat(g.get_state(0))
    finally:
        g.close()


def members_fused(status):
    """members at their own steps in one fused launch over two contexts"""
    import torch
    from mhm_gb300.model import MhmBatch, MhmGpu
    C = 48
    ctxs = []
    for i, (nr, nc, H, M) in enumerate([(20, 18, 5, 2), (10, 9, 2, 3)]):
        dom = synth.make_domain(nr, nc, H, l11_factor=2, seed=40 + i)
        l0 = synth.make_l0(dom, 2, seed=41 + i)
        g = MhmGpu(dom, n_members=M)
        g.mpr_setup(l0)
        g.mpr(params.random_gammas(M, 1, 0, 1, l0.n_geo, seed=42 + i))
        for m in range(M):
            g.init_states(m)
        f = synth.make_forcing(dom, C, seed=43 + i)
        g.set_meteo(1, *[torch.from_numpy(f[k]).cuda() for k in ("pre", "temp", "pet")], on_device=True)
        ctxs.append(g)
    batch = MhmBatch()
    try:
        out = []
        for r in range(2):
            q = [np.zeros((g.n_members, 1, C)) for g in ctxs]
            t0 = [np.array([1 + r * C if (m + r) % 2 == 0 else 0 for m in range(g.n_members)], np.int32)
                  for g in ctxs]
            batch.run_members(ctxs, t0, C, q)
            for g in ctxs:
                g.sync()
            out += [x.reshape(-1) for x in q]
        for g in ctxs:
            status.append(g.device_status())
        return np.concatenate(out), np.concatenate([_flat(g.get_state(0)) for g in ctxs])
    finally:
        batch.close()
        for g in ctxs:
            g.close()


def lai_series_mpr(status):
    """a monthly gridded LAI series regionalised on the device, PET case -1"""
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(14, 12, 3, l11_factor=2, seed=51, jul_start=2447893)
    l0 = synth.make_l0(dom, 2, seed=52)
    l0.lai_series = np.random.default_rng(53).uniform(0.2, 6.0, (3, l0.n_cells0))
    l0.gridded_lai = True
    gam = params.random_gammas(2, 1, -1, 1, l0.n_geo, seed=54)
    f = synth.make_forcing(dom, 24 * 70, seed=55)
    g = MhmGpu(dom, proc_pet=-1, n_members=2)
    try:
        g.set_lai_series(-2, 3)
        g.mpr_setup(l0)
        g.mpr(gam)
        for m in range(2):
            g.init_states(m)
        g.set_meteo(1, **f)
        q = np.concatenate([g.run(1, 24 * 35), g.run(24 * 35 + 1, 24 * 35)], axis=2)
        status.append(g.device_status())
        return q.reshape(-1), _flat(g.get_state(1))
    finally:
        g.close()


SCENARIOS = [ensemble_chunks, inflow_window, members_fused, lai_series_mpr]


def run_all():
    status = []
    res = {}
    for fn in SCENARIOS:
        q, s = fn(status)
        res[fn.__name__ + "_q"] = q
        res[fn.__name__ + "_s"] = s
    return res, status


if __name__ == "__main__":
    from mhm_gb300 import _lib
    from mhm_gb300.model import MhmGpu
    L = _lib.load()
    res, status = run_all()
    res["bounds_checked"] = np.array(L.mhm_bounds_checked())
    res["status_clean"] = np.array(all(s is None for s in status))
    # the reporting path: one failing test with no access behind it
    dom = synth.make_domain(8, 8, 2, l11_factor=2, seed=5)
    g = MhmGpu(dom)
    try:
        g.bounds_selftest()
        rep = g.device_status()
        res["selftest"] = np.array(rep if rep else (0, 0))
        res["after_selftest"] = np.array(g.device_status() is None)    # read and cleared
    finally:
        g.close()
    np.savez(sys.argv[1], **res)
    print("bounds-checked scenarios written", os.environ.get("MHM_BOUNDS_CHECK"))
