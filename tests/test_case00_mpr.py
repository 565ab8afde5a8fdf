"""The reference's own regression output pins the parameter regionalisation.

Fixture tests/golden/case00_mpr.npz (made by tests/golden/make_case00_mpr.py
from the reference's check/case_00: the test_domain basin at 500 m L0 /
24 km L1, 1475 soil types, 2 land-cover scenes, and the L1 effective
parameters the reference wrote to its restart file).  The oracle's hmath
build and the device MPR reproduce the reference's numbers bit for bit (all
36 parameter arrays of both scenes); the libm build is held to 1e-12, since
it follows whatever C library the host has."""
from pathlib import Path

import numpy as np
import pytest

from mhm_gb300 import params, synth
from oracle import oracle

FIX = Path(__file__).resolve().parent / "golden" / "case00_mpr.npz"
RTOL = 1e-12  # libm build; the hmath build and the device must match exactly
H = 2
# reference name in the restart file -> mhm_eff_params name
NAMES = {"fSealed": "fSealed", "alpha": "alpha", "degDayInc": "degDayInc", "degDayMax": "degDayMax",
         "degDayNoPre": "degDayNoPre", "fAsp": "fAsp", "karstLoss": "karstLoss", "kfastFlow": "kFastFlow",
         "kSlowFlow": "kSlowFlow", "kBaseFlow": "kBaseFlow", "kPerco": "kPerco", "tempThresh": "tempThresh",
         "unsatThresh": "unsatThresh", "sealedThresh": "sealedThresh", "maxInter": "maxInter",
         "fRoots": "fRoots", "soilMoistSat": "soilMoistSat", "soilMoistFC": "soilMoistFC",
         "wiltingPoint": "wiltingPoint", "soilMoistExp": "soilMoistExp"}
# written inside the reference's land-cover scene loop into scene 1: the last scene's values remain
LAST_SCENE = ("unsatThresh", "karstLoss")


def load_case():
    z = np.load(FIX)
    n0 = int(z["soil_id0"].size)
    mask = np.unpackbits(z["mask0"])[: int(z["n_mask0"])].astype(np.uint8)

    def l0_for(scene: int) -> synth.L0Maps:
        return synth.L0Maps(
            nrows0=int(z["nrows0"]), ncols0=int(z["ncols0"]), factor=int(z["factor"]), mask0=mask,
            l1_up=z["l1_up"], l1_down=z["l1_down"], l1_left=z["l1_left"], l1_right=z["l1_right"],
            l1_nsub=z["l1_nsub"], soil_id0=z["soil_id0"].astype(np.int32),
            lcover0=z["lcover0"][scene].astype(np.int32), geo_unit0=z["geo_unit0"].astype(np.int32),
            slope0=z["slope0"].astype(np.float64), aspect0=z["aspect0"].astype(np.float64),
            y0=np.full(n0, 49.5), lai_class0=z["lai_class0"].astype(np.int32), lai_lut=z["lai_lut"],
            soil_n_hor=z["soil_n_hor"], soil_n_till=z["soil_n_till"], soil_ud=z["soil_ud"], soil_ld=z["soil_ld"],
            soil_sand=z["soil_sand"], soil_clay=z["soil_clay"], soil_dbm=z["soil_dbm"],
            soil_rz_depth=z["soil_rz_depth"], geo_unit_list=z["geo_unit_list"], geo_unit_kar=z["geo_unit_kar"],
            horizon_depth=z["horizon_depth"].astype(np.float64), frac_sealed_city=float(z["frac_sealed_city"]))

    gold = {k[5:]: z[k] for k in z.files if k.startswith("gold_")}
    return l0_for, gold, z["gamma"], int(z["l1_up"].size)


def gold_for(gold, name, scene, n_scenes=2):
    g = gold[name]
    if name in LAST_SCENE:
        return None if scene != n_scenes - 1 else g[0]
    if g.shape[0] == 1:
        return g[0] if scene == 0 else None
    if name == "maxInter":
        return g.reshape(-1)
    return g[scene].reshape(-1)


def max_rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("kind", ["libm", "hmath"])
def test_oracle_mpr_reproduces_the_reference_case00(kind):
    l0_for, gold, gamma, n1 = load_case()
    off = np.array([0, 1, 9, 26, 27, 30, 35, 38, 43, 53, 53])
    worst = {}
    for scene in (0, 1):
        r = oracle.oracle_mpr(n1, H, l0_for(scene), gamma, off, 1, 0, kind)
        for gname, ename in NAMES.items():
            want = gold_for(gold, gname, scene)
            if want is None:
                continue
            got = r[ename]
            worst[gname] = max(worst.get(gname, 0.0), max_rel(got, want))
    tol = 0.0 if kind == "hmath" else RTOL
    bad = {k: v for k, v in worst.items() if not v <= tol}
    assert not bad, bad


def test_gamma_layout_of_the_case():
    off = params.layout(1, 0, 1, 10)
    assert list(off) == [0, 1, 9, 26, 27, 30, 35, 38, 43, 53, 53]


@pytest.mark.gpu
def test_gpu_mpr_reproduces_the_reference_case00():
    from mhm_gb300.model import MhmGpu
    l0_for, gold, gamma, n1 = load_case()
    dom = synth.make_domain(1, n1, H, l11_factor=1, seed=1)
    off = params.layout(1, 0, 1, 10)
    for scene in (0, 1):
        g = MhmGpu(dom, proc_soilmoist=1, proc_pet=0, n_members=1)
        try:
            l0 = l0_for(scene)
            g.mpr_setup(l0)
            g.mpr(gamma)
            got = g.get_eff_params(0)
        finally:
            g.close()
        ref = oracle.oracle_mpr(n1, H, l0, gamma, off, 1, 0, "hmath")
        for gname, ename in NAMES.items():
            assert np.array_equal(got[ename], ref[ename]), ename        # device == oracle, bit for bit
            want = gold_for(gold, gname, scene)
            if want is not None:
                assert np.array_equal(got[ename], want), (gname, max_rel(got[ename], want))
