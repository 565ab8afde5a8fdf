"""Contexts on two GPUs in one process: every context entry point makes the
context's own device current for the call and puts the caller's device back,
so a context works whatever device the caller has current and leaves that
choice alone.  Skips on machines with fewer than two GPUs."""
import numpy as np
import pytest

from mhm_gb300 import params, synth

pytestmark = pytest.mark.gpu


def test_contexts_on_two_devices_while_the_other_is_current():
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(16, 20, 3, 4, seed=5)
    l0 = synth.make_l0(dom, 2, seed=4)
    gam = params.default_gamma(1, 0, 1, l0.n_geo)
    f = synth.make_forcing(dom, 24 * 5, seed=7)
    out = []
    for dev in (0, 1):
        torch.cuda.set_device(1 - dev)
        g = MhmGpu(dom, device=dev)
        try:
            g.mpr_setup(l0)
            g.mpr(gam)
            g.init_states(0)
            g.set_meteo(1, **f)
            q = g.run(1, 24 * 5)
            st = g.get_state()
            assert torch.cuda.current_device() == 1 - dev
            out.append((q, st["soilMoist"]))
        finally:
            g.close()
        assert torch.cuda.current_device() == 1 - dev
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))
