"""The namelist reader and the run configuration taken from it.

The syntax cases are written here; the reader is also pinned to the
reference's own check-case namelists (the groups it reads, extracted by
tests/golden/make_namelist_excerpts.py into namelist_excerpts.json):
case_00's tables and parameter vector
equal the ones the case_00 fixtures hold (built by a separate parser in
tests/golden/make_case00_*.py), and case_04's and case_05's multi-domain
periods, resolutions and (inflow) gauges are read as their namelists state."""
import json
from pathlib import Path

import numpy as np
import pytest

from mhm_gb300 import namelist as nl

HERE = Path(__file__).resolve().parent
EXCERPTS = json.loads((HERE / "golden" / "namelist_excerpts.json").read_text())

TEXT = """
! a comment line
&mainconfig
    ndomains = 2   ! trailing comment
    resolution_hydrology(1:2) = 24000, 1.2d4
    name = 'a/b, c ! not a comment'
/
&time_periods
    warming_days(1:2) = 2*181
    eval_per(2)%ystart = 1991
    eval_per(1)%ystart = 1990 eval_per(1)%mstart = 7
/
&gauges
    gauge_id(1,1:2) = 398, 333
    gauge_id(2,1) = 45
    headwater(2,1) = .true.
    flags(1:3) = .false., T,
                 .t.
/
&geoparameter
GeoParam(1,:)  =  1.000,  1000.00,  100.0,  1,  1
GeoParam(2,:)  =  2.0, 3.0, -4.5e-1, 0, 1
/
"""


def test_syntax():
    g = nl.read(TEXT)
    assert nl.get(g, "mainconfig", "ndomains") == 2
    assert nl.get(g, "mainconfig", "resolution_hydrology") == [24000, 12000.0]
    assert nl.get(g, "mainconfig", "name") == "a/b, c ! not a comment"
    assert nl.get(g, "time_periods", "warming_days") == [181, 181]
    assert nl.array(g, "time_periods", "eval_per", "ystart") == {(1,): 1990, (2,): 1991}
    assert nl.array(g, "time_periods", "eval_per", "mstart") == {(1,): 7}
    assert nl.array(g, "gauges", "gauge_id") == {(1, 1): 398, (1, 2): 333, (2, 1): 45}
    assert nl.array(g, "gauges", "headwater") == {(2, 1): True}
    assert nl.get(g, "gauges", "flags") == [False, True, True]
    assert nl.array(g, "geoparameter", "geoparam")[(2, 3)] == -0.45
    assert [a.values[2] for a in g["geoparameter"]] == [100.0, -0.45]


def test_json_image_round_trip():
    g = nl.read(TEXT)
    h = nl.from_json(nl.to_json(g))
    for grp, key, comp in (("mainconfig", "resolution_hydrology", None), ("time_periods", "eval_per", "ystart"),
                           ("gauges", "gauge_id", None), ("gauges", "flags", None)):
        assert nl.array(h, grp, key, comp) == nl.array(g, grp, key, comp)


def test_unclosed_group_is_an_error():
    with pytest.raises(ValueError):
        nl.read("&a\n x = 1\n")


def test_case00_configuration_and_parameters():
    z = np.load(HERE / "golden" / "case00_run.npz")
    cfg = nl.run_config(EXCERPTS["case_00/mhm.nml"])
    assert cfg.process_case == [1, 1, 1, 1, 0, 1, 1, 1, 1, 0]
    assert (cfg.proc_sm, cfg.proc_pet, cfg.proc_rout) == (1, 0, 1)
    assert cfg.timestep == 1 and cfg.n_soil_horizons == 2 and cfg.soil_depth == [200.0]
    assert np.array_equal(cfg.evap_coeff, z["evap_coeff"])
    for k in ("prec", "pet", "temp"):
        assert np.array_equal(getattr(cfg, "fnight_" + k), z["fnight_" + k])
    assert cfg.frac_sealed_city_area == 0.6
    assert cfg.warming_days == [181] and cfg.eval_per == [(1990, 7, 1, 1991, 6, 30)]
    assert cfg.gauges == [[398]] and cfg.inflow_gauges == [[]]
    assert cfg.lcover_years == [(1981, 1990), (1991, 2000)]
    import test_case00_mpr as mpr_case
    gam = nl.gamma(EXCERPTS["case_00/mhm_parameter.nml"], 1, 0, 1)
    assert np.array_equal(np.array(gam), np.asarray(mpr_case.load_case()[2]))
    # the JSON image gives the same configuration
    g = nl.read(EXCERPTS["case_00/mhm.nml"])
    assert nl.run_config(nl.from_json(nl.to_json(g))) == cfg


def test_multi_domain_cases():
    c5 = nl.run_config(EXCERPTS["case_05/mhm.nml"])
    assert c5.n_domains == 3 and c5.gauges == [[398, 333]] * 3
    assert c5.inflow_gauges == [[(333, False)], [(333, True)], []]
    c4 = nl.run_config(EXCERPTS["case_04/mhm.nml"])
    assert c4.resolution_hydrology == [24000.0, 12000.0, 24000.0, 24000.0, 12000.0, 24000.0]
    assert c4.resolution_routing == [24000.0, 24000.0, 24000.0, 24000.0, 12000.0, 24000.0]
    assert c4.warming_days == [180, 180, 180, 360, 50, 0]
    assert c4.eval_per[1] == (1991, 1, 1, 1992, 12, 31)
    assert c4.gauges[2] == [] and c4.gauges[5] == [45]
