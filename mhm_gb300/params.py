"""Global parameter vectors (gamma) for the parameter regionalisation.

The rows below are the process blocks of mHM's parameter namelist
(mhm_parameter.nml: name, lower bound, upper bound, value, FLAG) for the
process cases this package runs; the vector is laid out process by process
in processMatrix order (src/MPR/mo_mpr_read_config.f90:390-990), the layout
`mhm_gamma_layout` reports.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

# (name, lower, upper, value, flag)
INTERCEPTION1 = [("canopyInterceptionFactor", 0.15, 0.40, 0.15, 1)]
SNOW1 = [
    ("snowTreshholdTemperature", -2.0, 2.0, 1.0, 1),
    ("degreeDayFactor_forest", 0.0001, 4.0, 1.5, 1),
    ("degreeDayFactor_impervious", 0.0, 1.0, 0.5, 1),
    ("degreeDayFactor_pervious", 0.0, 2.0, 0.5, 1),
    ("increaseDegreeDayFactorByPrecip", 0.1, 0.9, 0.5, 1),
    ("maxDegreeDayFactor_forest", 0.0, 8.0, 3.0, 1),
    ("maxDegreeDayFactor_impervious", 0.0, 8.0, 3.5, 1),
    ("maxDegreeDayFactor_pervious", 0.0, 8.0, 4.0, 1),
]
_SM_PTF = [
    ("orgMatterContent_forest", 0.0, 20.0, 3.4, 1),
    ("orgMatterContent_impervious", 0.0, 1.0, 0.1, 1),
    ("orgMatterContent_pervious", 0.0, 4.0, 0.6, 1),
    ("PTF_lower66_5_constant", 0.6462, 0.9506, 0.76, 1),
    ("PTF_lower66_5_clay", 0.0001, 0.0029, 0.0009, 1),
    ("PTF_lower66_5_Db", -0.3727, -0.1871, -0.264, 1),
    ("PTF_higher66_5_constant", 0.5358, 1.1232, 0.89, 1),
    ("PTF_higher66_5_clay", -0.0055, 0.0049, -0.001, 1),
    ("PTF_higher66_5_Db", -0.5513, -0.0913, -0.324, 1),
    ("PTF_Ks_constant", -1.2, -0.285, -0.585, 1),
    ("PTF_Ks_sand", 0.006, 0.026, 0.0125, 1),
    ("PTF_Ks_clay", 0.003, 0.013, 0.0063, 1),
    ("PTF_Ks_curveSlope", 60.96, 60.96, 60.96, 0),
]
_ROOTS_12 = [
    ("rootFractionCoefficient_forest", 0.9, 0.999, 0.97, 1),
    ("rootFractionCoefficient_impervious", 0.9, 0.95, 0.93, 1),
    ("rootFractionCoefficient_pervious", 0.001, 0.09, 0.02, 1),
    ("infiltrationShapeFactor", 1.0, 4.0, 1.75, 1),
]
_ROOTS_34 = [
    ("rootFractionCoefficient_forest", 0.97, 0.985, 0.975, 1),
    ("rootFractionCoefficient_impervious", 0.97, 0.985, 0.975, 1),
    ("rootFractionCoefficient_pervious", 0.97, 0.985, 0.975, 1),
    ("infiltrationShapeFactor", 1.0, 4.0, 1.75, 1),
    ("rootFractionCoefficient_sand", 0.001, 0.09, 0.09, 1),
    ("rootFractionCoefficient_clay", 0.9, 0.999, 0.98, 1),
    ("FCmin_glob", 0.1, 0.2, 0.15, 0),
    ("FCdelta_glob", 0.1, 0.4, 0.25, 0),
]
_JARVIS = [("jarvis_sm_threshold_c1", 0.0, 1.0, 0.5, 1)]
SOILMOISTURE = {1: _SM_PTF + _ROOTS_12, 2: _SM_PTF + _ROOTS_12 + _JARVIS,
                3: _SM_PTF + _ROOTS_34 + _JARVIS, 4: _SM_PTF + _ROOTS_34}
DIRECTRUNOFF1 = [("imperviousStorageCapacity", 0.0, 5.0, 0.5, 1)]
PET = {
    -1: [("PET_a_forest", 0.3, 1.3, 0.3, 1), ("PET_a_impervious", 0.3, 1.3, 0.8, 1),
         ("PET_a_pervious", 0.3, 1.3, 1.3, 1), ("PET_b", 0.0, 1.5, 1.5, 1), ("PET_c", -2.0, 0.0, -0.7, 1)],
    0: [("minCorrectionFactorPET", 0.7, 1.3, 0.9, 1), ("maxCorrectionFactorPET", 0.0, 0.2, 0.1, 1),
        ("aspectTresholdPET", 160.0, 200.0, 180.0, 1)],
    1: [("minCorrectionFactorPET", 0.7, 1.3, 0.93, 1), ("maxCorrectionFactorPET", 0.0, 0.2, 0.19, 1),
        ("aspectTresholdPET", 160.0, 200.0, 171.0, 1), ("HargreavesSamaniCoeff", 0.0016, 0.003, 0.0023, 1)],
}
INTERFLOW1 = [
    ("interflowStorageCapacityFactor", 75.0, 200.0, 85.0, 1),
    ("interflowRecession_slope", 0.0, 10.0, 7.0, 1),
    ("fastInterflowRecession_forest", 1.0, 3.0, 1.5, 1),
    ("slowInterflowRecession_Ks", 1.0, 30.0, 15.0, 1),
    ("exponentSlowInterflow", 0.05, 0.3, 0.125, 1),
]
PERCOLATION1 = [
    ("rechargeCoefficient", 0.0, 50.0, 35.0, 1),
    ("rechargeFactor_karstic", -5.0, 5.0, -1.0, 1),
    ("gain_loss_GWreservoir_karstic", 1.0, 1.0, 1.0, 0),
]
ROUTING = {0: [], 1: [
    ("muskingumTravelTime_constant", 0.31, 0.35, 0.325, 1),
    ("muskingumTravelTime_riverLength", 0.07, 0.08, 0.075, 1),
    ("muskingumTravelTime_riverSlope", 1.95, 2.1, 2.0, 1),
    ("muskingumTravelTime_impervious", 0.09, 0.11, 0.1, 1),
    ("muskingumAttenuation_riverSlope", 0.01, 0.5, 0.3, 1),
]}


def geo_rows(n_geo: int) -> list:
    return [(f"GeoParam({i + 1},:)", 1.0, 1000.0, 100.0, 1) for i in range(n_geo)]


def rows(proc_sm: int, proc_pet: int, proc_rout: int, n_geo: int) -> list:
    """Namelist rows in global-parameter order."""
    return (INTERCEPTION1 + SNOW1 + SOILMOISTURE[proc_sm] + DIRECTRUNOFF1 + PET[proc_pet] + INTERFLOW1 +
            PERCOLATION1 + ROUTING[proc_rout] + geo_rows(n_geo))


def layout(proc_sm: int, proc_pet: int, proc_rout: int, n_geo: int) -> np.ndarray:
    """Start offsets of processes 1..10 and the total, from the library."""
    from . import _lib
    L = _lib.load()
    out = np.zeros(11, np.int32)
    rc = L.mhm_gamma_layout(proc_sm, proc_pet, proc_rout, n_geo, out.ctypes.data_as(C.POINTER(C.c_int32)))
    if rc != 0:
        raise ValueError("no parameter layout for these process cases")
    return out


def offsets(proc_sm: int, proc_pet: int, proc_rout: int, n_geo: int) -> np.ndarray:
    """The same start offsets as `layout`, counted from the namelist blocks
    above without the library (for hosts that only run the CPU oracle)."""
    blocks = [INTERCEPTION1, SNOW1, SOILMOISTURE[proc_sm], DIRECTRUNOFF1, PET[proc_pet], INTERFLOW1,
              PERCOLATION1, ROUTING[proc_rout], geo_rows(n_geo)]
    out = np.zeros(11, np.int32)
    acc = 0
    for i, b in enumerate(blocks):
        out[i] = acc
        acc += len(b)
    out[9] = out[10] = acc   # process 10 (neutrons) has no parameters
    return out


def default_gamma(proc_sm: int = 1, proc_pet: int = 0, proc_rout: int = 1, n_geo: int = 4) -> np.ndarray:
    """The namelist's `value` column."""
    return np.array([r[3] for r in rows(proc_sm, proc_pet, proc_rout, n_geo)], np.float64)


def random_gammas(n: int, proc_sm: int = 1, proc_pet: int = 0, proc_rout: int = 1, n_geo: int = 4,
                  seed: int = 3) -> np.ndarray:
    """[n][n_gamma]: rows with FLAG = 1 uniform within their bounds, the others at their value
    (a calibration ensemble)."""
    rng = np.random.default_rng(seed)
    rr = rows(proc_sm, proc_pet, proc_rout, n_geo)
    lo = np.array([r[1] for r in rr])
    hi = np.array([r[2] for r in rr])
    val = np.array([r[3] for r in rr])
    flag = np.array([r[4] for r in rr], bool)
    g = np.tile(val, (n, 1))
    u = rng.uniform(size=(n, len(rr)))
    g[:, flag] = (lo + u * (hi - lo))[:, flag]
    return np.ascontiguousarray(g)
