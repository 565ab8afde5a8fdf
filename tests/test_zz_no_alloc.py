"""mhm_mpr_noalloc: the parameter regionalisation of one member with its
per-call data in the library's static device scratch, called through the C
ABI and compared with mhm_mpr on the same inputs, two calls in a row.

Both entry points launch the same kernels on the same inputs, so every
effective parameter (including the LAI-based PET correction of PET case -1,
which uses the third region of the scratch) and the Muskingum coefficients
must be BIT-IDENTICAL.

The file name sorts last so that the test also runs after every other test
in one session (the scratch is a process-wide device array)."""
import ctypes as C

import numpy as np
import pytest

from mhm_gb300 import params, synth

_dp = C.POINTER(C.c_double)


def _bitwise(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("proc_pet", [0, -1])
def test_mpr_noalloc_matches_mpr_two_calls_in_a_row(proc_pet):
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(12, 10, 3, l11_factor=2, seed=1)
    l0 = synth.make_l0(dom, 4, seed=4, holes=0.1)     # class LAI (12 classes): petLAIcorFactor from the table
    gam = params.random_gammas(2, 1, proc_pet, 1, l0.n_geo, seed=21)
    g = MhmGpu(dom, proc_soilmoist=1, proc_pet=proc_pet, n_members=2)
    try:
        g.mpr_setup(l0)
        for call in range(2):
            gm = np.ascontiguousarray(gam[call])
            g.mpr(gm, member0=0)                                   # existing entry point
            rc = g.L.mhm_mpr_noalloc(g.ctx, 1, gm.ctypes.data_as(_dp), gm.size)
            assert rc == 0, g.L.mhm_last_error(g.ctx)
            want, got = g.get_eff_params(0), g.get_eff_params(1)
            if proc_pet == -1:
                assert "petLAIcorFactor" in want and np.all(want["petLAIcorFactor"] > 0)
            for name in want:
                assert _bitwise(got[name], want[name]), (call, name)
            st0, st1 = g.get_state(0), g.get_state(1)
            assert _bitwise(st1["C1"], st0["C1"]) and _bitwise(st1["C2"], st0["C2"]), call
    finally:
        g.close()


@pytest.mark.gpu
def test_mpr_noalloc_writes_a_gridded_lai_series():
    """with a gridded LAI series the LAI-indexed parameters go to the series,
    bit-identical to mhm_mpr's"""
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(12, 10, 3, l11_factor=2, seed=1)
    l0 = synth.make_l0(dom, 4, seed=4)
    l0.lai_series = np.random.default_rng(5).uniform(0.2, 6.0, (7, l0.n_cells0))
    l0.gridded_lai = True
    gm = np.ascontiguousarray(params.random_gammas(1, 1, -1, 1, l0.n_geo, seed=22)[0])
    g = MhmGpu(dom, proc_soilmoist=1, proc_pet=-1, n_members=2)
    try:
        g.set_lai_series(-3, 7)
        g.mpr_setup(l0)
        g.mpr(gm, member0=0)
        rc = g.L.mhm_mpr_noalloc(g.ctx, 1, gm.ctypes.data_as(_dp), gm.size)
        assert rc == 0, g.L.mhm_last_error(g.ctx)
        want, got = g.get_lai_params(7, 0), g.get_lai_params(7, 1)
        assert np.all(want[0] > 0) and np.all(want[1] > 0)
        for a, b in zip(want[:2], got[:2]):
            assert _bitwise(a, b)
    finally:
        g.close()


@pytest.mark.gpu
def test_mpr_noalloc_rejects_tables_beyond_the_scratch():
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(4, 4, 6, l11_factor=2, seed=1)
    # 1000 soil types x 3 land covers x (5*6+4) doubles > 65,536
    l0 = synth.make_l0(dom, 2, seed=4, n_soil=1000)
    g = MhmGpu(dom, proc_soilmoist=1, proc_pet=0, n_members=1)
    try:
        g.mpr_setup(l0)
        gm = params.default_gamma(1, 0, 1, l0.n_geo)
        rc = g.L.mhm_mpr_noalloc(g.ctx, 0, gm.ctypes.data_as(_dp), gm.size)
        assert rc != 0
        assert b"scratch" in g.L.mhm_last_error(g.ctx)
        g.mpr(gm)   # the allocating entry point handles it
    finally:
        g.close()
