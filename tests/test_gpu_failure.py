"""Per-member failure detection on the device: the cell chain flags a member
whose total runoff or final states are NaN/Inf (integer test of the
exponent bits), mhm_member_status reports MHM_ERR_NAN for exactly that
member and clears the flags, and the other members' results are the ones
they give without the bad member."""
import numpy as np
import pytest

from mhm_gb300 import params, synth
from mhm_gb300._lib import MHM_ERR_NAN

pytestmark = pytest.mark.gpu


def _ctx(dom, l0, gam, M):
    from mhm_gb300.model import MhmGpu
    g = MhmGpu(dom, n_members=M)
    g.mpr_setup(l0)
    g.mpr(gam[:M])
    for m in range(M):
        g.init_states(m)
    return g


def test_nonfinite_member_is_flagged_alone():
    dom = synth.make_domain(16, 12, 3, l11_factor=2, seed=1)
    l0 = synth.make_l0(dom, 2, seed=4)
    gam = params.random_gammas(3, 1, 0, 1, l0.n_geo, seed=8)
    f = synth.make_forcing(dom, 48, seed=2)
    clean = _ctx(dom, l0, gam, 3)
    poisoned = _ctx(dom, l0, gam, 3)
    try:
        st = poisoned.get_state(1)
        st["unsatSTW"][5] = np.nan                      # a corrupt warm start of member 1
        poisoned.set_state({"unsatSTW": st["unsatSTW"]}, 1)
        for g in (clean, poisoned):
            g.set_meteo(1, **f)
        qc = clean.run(1, 48)
        qp = poisoned.run(1, 48)
        assert list(clean.member_status()) == [0, 0, 0]
        assert list(poisoned.member_status()) == [0, MHM_ERR_NAN, 0]
        assert list(poisoned.member_status()) == [0, 0, 0]    # read-and-clear
        assert not np.all(np.isfinite(qp[1]))
        for m in (0, 2):
            assert np.array_equal(qp[m], qc[m]) and np.all(np.isfinite(qp[m]))
    finally:
        clean.close()
        poisoned.close()


def test_nonfinite_forcing_flags_every_member_that_reads_it():
    dom = synth.make_domain(16, 12, 3, l11_factor=2, seed=1)
    l0 = synth.make_l0(dom, 2, seed=4)
    gam = params.random_gammas(2, 1, 0, 1, l0.n_geo, seed=9)
    f = synth.make_forcing(dom, 48, seed=2)
    f["pre"][10, 7] = np.inf
    g = _ctx(dom, l0, gam, 2)
    try:
        g.set_meteo(1, **f)
        g.run(1, 48)
        assert list(g.member_status()) == [MHM_ERR_NAN, MHM_ERR_NAN]
    finally:
        g.close()
