#!/usr/bin/env python3
"""Write pfunit_kats.json: the known-answer cases of the reference's pFUnit
tests (src/tests/*.pf) for the hot-path routines, transcribed as data.

Each case cites the .pf line of its call and of its expected values.  When
run with the reference tree available (argument: its root directory), the
script also checks that every number of every case appears on the cited
lines, so the transcription can be re-verified; the JSON it writes is what
tests/test_oracle_kats.py reads (the reference tree is not needed there).

    python make_pfunit_kats.py [REFERENCE_ROOT]
"""
import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
T = 0.001  # tolerance t of every .pf file

CASES = [
    # canopy_interc(pet, interc_max, precip, interc[inout]) -> interc, throughfall, evap_canopy
    dict(routine="canopy_interc", src="src/tests/test_canopy_interc.pf", call=27,
         args=[0.1, 0.45, 0.39], inout={"interc": 0.345},
         expect={"interc": 0.35, "throughfall": 0.285, "evap_canopy": 0.1}),
    dict(routine="canopy_interc", src="src/tests/test_canopy_interc.pf", call=37,
         args=[0.1, 0.45, -0.39], inout={"interc": 0.345},
         expect={"interc": 0.0, "throughfall": 0.0, "evap_canopy": -0.045}),
    dict(routine="canopy_interc", src="src/tests/test_canopy_interc.pf", call=47,
         args=[0.1, -0.45, 0.39], inout={"interc": 0.345},
         expect={"interc": 0.0, "throughfall": 1.185, "evap_canopy": -0.45}),
    # snow_accum_melt(incr, max, noprec, prec, temp, thresh, thrfall, snow_pack[inout]) -> ...
    dict(routine="snow_accum_melt", src="src/tests/test_snow_accum_melt.pf", call=32,
         args=[0.5, 0.232, 0.078, 0.208, 8.31, 1.0, 0.195], inout={"snow_pack": 0.0},
         expect={"snow_pack": 0.0, "deg_day": 0.182, "melt": 0.0, "prec_effect": 0.195, "rain": 0.195, "snow": 0.0}),
    dict(routine="snow_accum_melt", src="src/tests/test_snow_accum_melt.pf", call=48,
         args=[0.5, 0.232, 0.078, 0.208, -8.31, 1.0, 0.195], inout={"snow_pack": 0.0},
         expect={"snow_pack": 0.195, "deg_day": 0.182, "melt": 0.0, "prec_effect": 0.0, "rain": 0.0, "snow": 0.195}),
    dict(routine="snow_accum_melt", src="src/tests/test_snow_accum_melt.pf", call=65,
         args=[0.5, 0.232, 0.078, 0.208, 3.0, 1.0, 0.195], inout={"snow_pack": 0.3},
         expect={"snow_pack": 0.0, "deg_day": 0.182, "melt": 0.3, "prec_effect": 0.495, "rain": 0.195, "snow": 0.0}),
    dict(routine="snow_accum_melt", src="src/tests/test_snow_accum_melt.pf", call=83,
         args=[0.5, 0.232, 0.232, 0.208, 3.0, 1.0, 0.195], inout={"snow_pack": 0.6},
         expect={"snow_pack": 0.136, "deg_day": 0.232, "melt": 0.464, "prec_effect": 0.659, "rain": 0.195, "snow": 0.0}),
    # soil_moisture(case, fsealed, thresh_sealed, pet, evap_coeff, sat[], roots[], fc[], pw[], exp[], c1,
    #               aet_canopy, prec_effec, runoff_sealed[inout], storage_sealed[inout], infil[], sm[inout])
    dict(routine="soil_moisture", src="src/tests/test_soil_moisture.pf", call=42,
         args=[2, 0.03, 0.5, 0.3, 1.0, [91.0, 65.0], [0.6, 0.6], [67.0, 67.0], [21.2, 21.2], [2.2, 2.2], 0.5, 0.0, 0.0],
         inout={"storage_sealed": 0.0, "soil_moist": [43.0, 70.0]},
         expect={"runoff_sealed": 0.0, "storage_sealed": 0.0, "infiltration": [0.0, 0.0],
                 "soil_moist": [42.887, 69.887], "aet": [0.112, 0.112], "aet_sealed": 0.0}),
    dict(routine="soil_moisture", src="src/tests/test_soil_moisture.pf", call=78,
         args=[1, 0.03, 0.0, 0.3, 1.0, [1.0], [0.6], [0.0], [5.0], [2.2], 0.5, 0.5, 10.0],
         inout={"storage_sealed": 0.5, "soil_moist": [0.0]},
         expect={"runoff_sealed": 10.5, "storage_sealed": 0.0, "infiltration": [9.0],
                 "soil_moist": [1.0], "aet": [0.0], "aet_sealed": 0.0}),
    dict(routine="soil_moisture", src="src/tests/test_soil_moisture.pf", call=101,
         args=[1, 0.03, 0.5, 0.3, 1.0, [0.0], [0.6], [0.0], [5.0], [2.2], 0.5, 0.5, 1.0],
         inout={"storage_sealed": 1.0, "soil_moist": ["0.5*eps"]},
         expect={"runoff_sealed": 1.5, "storage_sealed": 0.5, "infiltration": [1.0],
                 "soil_moist": ["eps"], "aet": [0.0], "aet_sealed": 0.0}),
    dict(routine="feddes_et_reduction", src="src/tests/test_soil_moisture.pf", call=129,
         args=[38.5, 77.0, 43.6, 0.6], expect={"result": 0.0}),
    dict(routine="feddes_et_reduction", src="src/tests/test_soil_moisture.pf", call=134,
         args=[35.5, 71.1, 33.0, 0.618], expect={"result": 0.04}),
    dict(routine="feddes_et_reduction", src="src/tests/test_soil_moisture.pf", call=139,
         args=[35.5, 35.5, 33.0, 0.618], expect={"result": 0.618}),
    dict(routine="jarvis_et_reduction", src="src/tests/test_soil_moisture.pf", call=151,
         args=[48.1, 92.6, 32.2, 0.6, 0.5], expect={"result": 0.315}),
    dict(routine="jarvis_et_reduction", src="src/tests/test_soil_moisture.pf", call=161,
         args=[128.4, 319.0, 144.5, 0.4, 0.5], expect={"result": 0.0}),
    dict(routine="jarvis_et_reduction", src="src/tests/test_soil_moisture.pf", call=166,
         args=[91.3, 50.5, 38.2, 0.6, 0.5], expect={"result": 0.6}),
    # runoff_unsat_zone(k1, kp, k0, alpha, karst, pefec_soil, thresh, sat[inout], unsat[inout]) -> slow, fast, perc
    dict(routine="runoff_unsat_zone", src="src/tests/test_runoff.pf", call=32,
         args=[1.2417, 1.4312, 3.547, 0.285, 1.0, 0.0, 17.926], inout={"sat_storage": 35.304, "unsat_storage": 2.27},
         expect={"sat_storage": 35.304, "unsat_storage": 0.0, "slow_interflow": 2.27, "fast_interflow": 0.0,
                 "perc": 0.0}),
    dict(routine="runoff_unsat_zone", src="src/tests/test_runoff.pf", call=48,
         args=[1.2417, 1.4312, 3.547, 0.285, 1.0, 20.0, 17.926], inout={"sat_storage": 35.304, "unsat_storage": 2.27},
         expect={"sat_storage": 35.304, "unsat_storage": 0.0, "slow_interflow": 6.862, "fast_interflow": 15.408,
                 "perc": 0.0}),
    dict(routine="runoff_unsat_zone", src="src/tests/test_runoff.pf", call=64,
         args=[1.2417, 1.4312, 3.547, 0.285, 1.0, 0.0, 17.926], inout={"sat_storage": 35.304, "unsat_storage": -2.27},
         expect={"sat_storage": 32.055, "unsat_storage": 0.979, "slow_interflow": 0.0, "fast_interflow": 0.0,
                 "perc": -3.249}),
    dict(routine="runoff_sat_zone", src="src/tests/test_runoff.pf", call=84,
         args=[0.000417], inout={"sat_storage": 17.0}, expect={"sat_storage": 16.992, "baseflow": 0.007}),
    dict(routine="runoff_sat_zone", src="src/tests/test_runoff.pf", call=92,
         args=[0.000417], inout={"sat_storage": -17.0}, expect={"sat_storage": 0.0, "baseflow": 0.0}),
    dict(routine="L1_total_runoff", src="src/tests/test_runoff.pf", call=105,
         args=[0.0284, 0.0, 5.0, 5.365, 0.0], expect={"result": 10.07}),
    # PET (src/mHM/mo_pet.f90)
    dict(routine="pet_hargreaves", src="src/tests/test_pet.pf", call=24,
         args=[0.8, 17.8, 12.0, 20.0, 8.0, 23.1637, 150], expect={"result": 1349.437}),
    dict(routine="pet_priestly", src="src/tests/test_pet.pf", call=35,
         args=[1.26, 200.0, 10.0], expect={"result": 4.978}),
    dict(routine="pet_priestly", src="src/tests/test_pet.pf", call=39,
         args=[1.26, 0.0, 10.0], expect={"result": 0.0}),
    dict(routine="pet_penman", src="src/tests/test_pet.pf", call=50,
         args=[200.0, 10.0, 1.7, 60.0, 70.0, 1.0, 1.0], expect={"result": 1.074}),
    dict(routine="extraterr_rad_approx", src="src/tests/test_pet.pf", call=65,
         args=[150, "deg2rad*23.1637"], expect={"result": 16.34}),
    dict(routine="slope_satpressure", src="src/tests/test_pet.pf", call=76,
         args=[10.0], expect={"result": 0.082}),
    dict(routine="sat_vap_pressure", src="src/tests/test_pet.pf", call=87,
         args=[10.0], expect={"result": 1.228}),
    # temporal disaggregation (src/meteo/mo_meteo_temporal_tools.f90)
    dict(routine="temporal_disagg_meteo_weights", src="src/tests/test_meteo_temporal_tools.pf", call=26,
         args=[[2.74, 3.32], 0.3, 0.0], expect={"result": [0.822, 0.996]}),
    dict(routine="temporal_disagg_meteo_weights", src="src/tests/test_meteo_temporal_tools.pf", call=31,
         args=[[2.74, 3.32], 0.3, 0.5], expect={"result": [0.472, 0.646]}),
    dict(routine="temporal_disagg_flux_daynight", src="src/tests/test_meteo_temporal_tools.pf", call=44,
         args=[[1, 0, 1], [24.0, 24.0, 1.0], 2.74, 0.9, 0.1], expect={"result": [0.2055, 0.0228, 2.74]}),
    dict(routine="temporal_disagg_state_daynight", src="src/tests/test_meteo_temporal_tools.pf", call=58,
         args=[[1, 0, 1, 0, 1], [24.0, 24.0, 24.0, 24.0, 1.0], 2.74, 0.9, 0.1, [0, 0, 1, 1, 0]],
         expect={"result": [4.932, 0.548, 3.64, 2.84, 2.74]}),
]


def _numbers(obj):
    if isinstance(obj, (list, tuple)):
        for x in obj:
            yield from _numbers(x)
    elif isinstance(obj, dict):
        for x in obj.values():
            yield from _numbers(x)
    elif isinstance(obj, bool):
        return
    elif isinstance(obj, (int, float)):
        yield obj


def verify(root: Path) -> int:
    """Every number of a case must appear within the 45 lines before and the
    6 lines after its cited call; returns the number of unmatched values."""
    missing = 0
    for c in CASES:
        lines = (root / c["src"]).read_text().splitlines()
        nums = set()
        for ln in range(max(1, c["call"] - 45), min(len(lines), c["call"] + 6) + 1):
            for tok in re.findall(r"-?\d+\.?\d*(?:[eE][-+]?\d+)?", lines[ln - 1]):
                try:
                    nums.add(round(float(tok), 9))
                except ValueError:
                    pass
        for v in _numbers({"a": c["args"], "i": c.get("inout", {}), "e": c["expect"]}):
            if round(float(v), 9) not in nums and v not in (0, 1, 0.0, 1.0):
                missing += 1
                print(f"{c['src']}:{c['call']}: {v} not found on the cited lines")
    return missing


def main():
    out = {"tolerance": T, "source": "mHM src/tests/*.pf (pFUnit), transcribed", "cases": CASES}
    (HERE / "pfunit_kats.json").write_text(json.dumps(out, indent=1))
    if len(sys.argv) > 1:
        bad = verify(Path(sys.argv[1]))
        print("verification:", "ok" if bad == 0 else f"{bad} values unmatched")
        sys.exit(1 if bad else 0)


if __name__ == "__main__":
    main()
