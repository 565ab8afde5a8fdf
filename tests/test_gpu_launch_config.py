"""Launch configuration and the autotuner's knobs (register variant, routing
sub-chunk, time-chunk length) change how the work is launched, never the
results: every configuration gives the discharge and states of the default
one bit for bit, and the autotuner leaves the states as it found them."""
import numpy as np
import pytest

from mhm_gb300 import synth

pytestmark = pytest.mark.gpu


def _run(dom, p, f, T, cfg=None, tune=None):
    from mhm_gb300.model import MhmGpu
    g = MhmGpu(dom, n_members=2)
    try:
        g.prepare([p, p], synth.ROUTING_PARAMS_DEFAULT)
        g.set_meteo(1, **f)
        info = None
        if cfg:
            g.set_launch_config(**cfg)
            assert g.get_launch_config() == cfg
        if tune:
            info = g.autotune_ex(1, T, tune)
            assert info["chunk_steps"] in tune
        q = g.run(1, T)
        return q, g.get_state(1), info
    finally:
        g.close()


def test_configurations_give_identical_results():
    dom = synth.make_domain(24, 20, 3, 4, seed=3)
    p = synth.make_eff_params(dom, seed=4)
    T = 96
    f = synth.make_forcing(dom, T, seed=5)
    q0, s0, _ = _run(dom, p, f, T)
    for cfg in ({"cell_blocks_per_sm": 8, "route_sub_steps": 16, "chunk_steps": 24, "route_cluster": 0},
                {"cell_blocks_per_sm": 6, "route_sub_steps": 3, "chunk_steps": 40, "route_cluster": 0},
                {"cell_blocks_per_sm": 4, "route_sub_steps": 1, "chunk_steps": 0, "route_cluster": 0},
                {"cell_blocks_per_sm": 8, "route_sub_steps": 4, "chunk_steps": 40, "route_cluster": 16},
                {"cell_blocks_per_sm": 4, "route_sub_steps": 16, "chunk_steps": 0, "route_cluster": 8},
                {"cell_blocks_per_sm": 6, "route_sub_steps": 3, "chunk_steps": 24, "route_cluster": 4}):
        q, s, _ = _run(dom, p, f, T, cfg=cfg)
        assert np.array_equal(q, q0), cfg
        for k in s0:
            assert np.array_equal(s[k], s0[k]), (cfg, k)
    q, s, info = _run(dom, p, f, T, tune=[48, 96])
    assert len(info["trial_ms"]) == 18
    assert np.array_equal(q, q0)
    for k in s0:
        assert np.array_equal(s[k], s0[k]), k


def test_route_autotuner_keeps_results():
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(24, 20, 3, 4, seed=3)
    p = synth.make_eff_params(dom, seed=4)
    T = 96
    f = synth.make_forcing(dom, T, seed=5)
    q0, s0, _ = _run(dom, p, f, T)
    g = MhmGpu(dom, n_members=2)
    try:
        g.prepare([p, p], synth.ROUTING_PARAMS_DEFAULT)
        g.set_meteo(1, **f)
        info = g.autotune_route(1, T)
        assert info["route_cluster"] in (0, 4, 8, 16)
        assert len(info["route_trial_ms"]) == 4 and min(info["route_trial_ms"]) > 0
        assert g.get_launch_config()["route_cluster"] == info["route_cluster"]
        q = g.run(1, T)
        s = g.get_state(1)
    finally:
        g.close()
    assert np.array_equal(q, q0)
    for k in s0:
        assert np.array_equal(s[k], s0[k]), k
