"""The oracle against the reference's own known-answer tests (pFUnit files
src/tests/*.pf, transcribed in tests/golden/pfunit_kats.json by
tests/golden/make_pfunit_kats.py), at the reference's tolerance t = 0.001,
for both elementary-function builds."""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

KATS = json.loads((Path(__file__).parent / "golden" / "pfunit_kats.json").read_text())
EPS = np.finfo(np.float64).eps
D = C.c_double


def _val(v):
    if isinstance(v, str):
        return {"eps": EPS, "0.5*eps": 0.5 * EPS, "deg2rad*23.1637": math.pi / 180.0 * 23.1637}[v]
    return v


def _arr(v):
    return np.ascontiguousarray([_val(x) for x in v], np.float64)


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def run_case(L, c):
    r, a = c["routine"], [(_val(x) if not isinstance(x, list) else x) for x in c["args"]]
    io = c.get("inout", {})
    if r == "canopy_interc":
        interc, thr, ev = D(io["interc"]), D(), D()
        L.ora_canopy_interc(*a, C.byref(interc), C.byref(thr), C.byref(ev))
        return {"interc": interc.value, "throughfall": thr.value, "evap_canopy": ev.value}
    if r == "snow_accum_melt":
        sp = D(io["snow_pack"])
        out = [D() for _ in range(5)]
        L.ora_snow_accum_melt(*a, C.byref(sp), *[C.byref(o) for o in out])
        return dict(zip(["snow_pack", "deg_day", "melt", "prec_effect", "rain", "snow"],
                        [sp.value] + [o.value for o in out]))
    if r == "soil_moisture":
        case, fs, ths, pet, ec, sat, fr, fc, pw, ex, c1, aetc, pe = a
        nH = len(sat)
        sat, fr, fc, pw, ex = (_arr(x) for x in (sat, fr, fc, pw, ex))
        rs, ss, aets = D(0.0), D(io["storage_sealed"]), D()
        inf = np.zeros(nH)
        sm = _arr(io["soil_moist"])
        aet = np.zeros(nH)
        L.ora_soil_moisture(case, nH, fs, ths, pet, ec, _p(sat), _p(fr), _p(fc), _p(pw), _p(ex), c1, aetc, pe,
                            C.byref(rs), C.byref(ss), _p(inf), _p(sm), _p(aet), C.byref(aets))
        return {"runoff_sealed": rs.value, "storage_sealed": ss.value, "infiltration": list(inf),
                "soil_moist": list(sm), "aet": list(aet), "aet_sealed": aets.value}
    if r == "feddes_et_reduction":
        return {"result": L.ora_feddes_et_reduction(*a)}
    if r == "jarvis_et_reduction":
        return {"result": L.ora_jarvis_et_reduction(*a)}
    if r == "runoff_unsat_zone":
        sat, uns = D(io["sat_storage"]), D(io["unsat_storage"])
        sl, fa, pe = D(), D(), D()
        L.ora_runoff_unsat_zone(*a, C.byref(sat), C.byref(uns), C.byref(sl), C.byref(fa), C.byref(pe))
        return {"sat_storage": sat.value, "unsat_storage": uns.value, "slow_interflow": sl.value,
                "fast_interflow": fa.value, "perc": pe.value}
    if r == "runoff_sat_zone":
        sat, bf = D(io["sat_storage"]), D()
        L.ora_runoff_sat_zone(a[0], C.byref(sat), C.byref(bf))
        return {"sat_storage": sat.value, "baseflow": bf.value}
    if r == "L1_total_runoff":
        return {"result": L.ora_L1_total_runoff(*a)}
    if r == "pet_hargreaves":
        return {"result": L.ora_pet_hargreaves(*a)}
    if r == "pet_priestly":
        return {"result": L.ora_pet_priestly(*a)}
    if r == "pet_penman":
        return {"result": L.ora_pet_penman(*a)}
    if r == "extraterr_rad_approx":
        return {"result": L.ora_extraterr_rad_approx(int(a[0]), a[1])}
    if r == "slope_satpressure":
        return {"result": L.ora_slope_satpressure(*a)}
    if r == "sat_vap_pressure":
        return {"result": L.ora_sat_vap_pressure(*a)}
    if r == "temporal_disagg_meteo_weights":
        vals, w, corr = a
        return {"result": [L.ora_disagg_meteo_weights(v, w, corr) for v in vals]}
    if r == "temporal_disagg_flux_daynight":
        isday, nts, v, fd, fn = a
        return {"result": [L.ora_disagg_flux_daynight(d, n, v, fd, fn) for d, n in zip(isday, nts)]}
    if r == "temporal_disagg_state_daynight":
        isday, nts, v, fd, fn, addc = a
        return {"result": [L.ora_disagg_state_daynight(d, n, v, fd, fn, ac) for d, n, ac in zip(isday, nts, addc)]}
    raise KeyError(r)


@pytest.mark.parametrize("kind", ["hmath", "libm"])
@pytest.mark.parametrize("i", range(len(KATS["cases"])))
def test_pfunit_kat(kind, i, ora_hmath, ora_libm):
    L = ora_hmath if kind == "hmath" else ora_libm
    c = KATS["cases"][i]
    got = run_case(L, c)
    for k, exp in c["expect"].items():
        g = np.atleast_1d(np.asarray(got[k], np.float64))
        e = np.atleast_1d(np.asarray([_val(x) for x in (exp if isinstance(exp, list) else [exp])], np.float64))
        assert np.allclose(g, e, rtol=0, atol=KATS["tolerance"]), f"{c['src']}:{c['call']} {k}: {g} vs {e}"


def test_all_routines_covered():
    names = {c["routine"] for c in KATS["cases"]}
    assert {"canopy_interc", "snow_accum_melt", "soil_moisture", "runoff_unsat_zone", "runoff_sat_zone",
            "L1_total_runoff", "pet_hargreaves", "extraterr_rad_approx", "temporal_disagg_flux_daynight"} <= names
