"""Cell water balance closes on the GPU to 1e-12 relative.

Per cell and step (the mosaic of L1_total_runoff, src/mHM/mo_runoff.f90:
248-274): storage S = interception + snow + fSealed * sealed storage
+ (1 - fSealed) * (soil moisture of all horizons + unsaturated + saturated),
and dS = P - aET - Q - karst loss, with aET the area-weighted canopy, sealed
and soil evapotranspiration and the karst loss (1 - fSealed) * perc *
(1 - karstLoss).  Checked step by step (one-step calls with states read back)
and over a multi-day run, for soil-moisture cases 1-4, relative to the
largest of the storages and flux sums involved."""
import numpy as np
import pytest

from mhm_gb300 import params, synth

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _storage(st, p, N, H):
    fs = p["fSealed"]
    sm = st["soilMoist"].reshape(H, N).sum(0)
    return st["interc"] + st["snowpack"] + fs * st["sealSTW"] + (1.0 - fs) * (sm + st["unsatSTW"] + st["satSTW"])


def _model(proc_sm):
    from mhm_gb300.model import MhmGpu
    dom = synth.make_domain(14, 12, 4, l11_factor=2, seed=1)
    l0 = synth.make_l0(dom, 2, seed=4)
    g = MhmGpu(dom, proc_soilmoist=proc_sm, proc_pet=0, n_members=2)
    g.mpr_setup(l0)
    g.mpr(params.random_gammas(2, proc_sm, 0, 1, l0.n_geo, seed=9))
    for m in range(2):
        g.init_states(m)
    return dom, g


@pytest.mark.parametrize("proc_sm", [1, 2, 3, 4])
def test_water_balance_closes_per_step_and_over_a_run(proc_sm):
    dom, g = _model(proc_sm)
    N, H = dom.n_cells, dom.n_horizons
    T = 48
    f = synth.make_forcing(dom, T, seed=2, gamma_theta=4.0)
    try:
        g.set_meteo(1, f["pre"], f["temp"], f["pet"])
        g.run(1, 1)       # step 1 resets SM to 0.5 FC: start the balance after it
        g.enable_outputs(total_runoff=True)
        g.enable_fluxes(True)
        p = [g.get_eff_params(m) for m in range(2)]
        s0 = [_storage(g.get_state(m), p[m], N, H) for m in range(2)]
        prev = list(s0)
        sums = [np.zeros(N) for _ in range(2)]
        scale = [np.zeros(N) for _ in range(2)]
        for tt in range(2, T + 1):          # per-step closure
            g.run(tt, 1)
            tro, _ = g.get_outputs()
            aet, loss = g.get_fluxes()
            for m in range(2):
                s1 = _storage(g.get_state(m), p[m], N, H)
                flux = f["pre"][tt - 1] - aet[0, m] - tro[0, m] - loss[0, m]
                mag = np.maximum.reduce([np.abs(prev[m]), np.abs(s1), np.abs(f["pre"][tt - 1]), np.abs(aet[0, m]),
                                         np.abs(tro[0, m])]) + 1e-300
                err = np.abs((s1 - prev[m]) - flux) / mag
                assert err.max() < TOL, (tt, m, err.max())
                sums[m] += flux
                scale[m] = np.maximum(scale[m], mag)
                prev[m] = s1
        for m in range(2):                  # closure over the whole run
            err = np.abs((prev[m] - s0[m]) - sums[m]) / scale[m]
            assert err.max() < T * TOL, (m, err.max())
    finally:
        g.close()
