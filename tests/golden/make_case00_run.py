#!/usr/bin/env python3
"""Build tests/golden/case00_run.npz: everything besides the parameter
regionalisation that the reference's regression case check/case_00 feeds its
time loop, and what the loop produced.

Inputs (from the reference tree at REF): daily meteo (test_domain
pre/tavg/pet netCDF-4, L2 = L1 = 24 km) for the simulated period 1990-01-01
.. 1991-06-30 (181 warm-up days + the evaluation year), the L11 network mRM
built (L11_fromN/toN/netPerm/length/slope, the floodplain impervious
fraction per land-cover scene, cell areas, the gauge node) from
b1_mRM_restart_001.nc (with the L11 mask and flow directions it was built
from), and case_00's mhm.nml meteo tables.  Outputs: the
daily simulated discharge of b1_daily_discharge.out and the final states of
both restart files.  Cell arrays are packed column-major over mHM's (x, y)
L1 mask, i.e. in the row-major order of the north-first grids.

Also writes case10_gold.npz, case12_gold.npz and case09_gold.npz: check/
case_10 and case_12 run the same inputs with soil-moisture cases 3 and 4 and
the LAI-based PET correction (processCase(5) = -1), case_09 with
Hargreaves-Samani PET (daily tmin/tmax) and adaptive routing case 2; their
parameter vectors (from their mhm_parameter.nml), L1 parameters, final
states and daily discharge.

Every case also gets its aggregated outputs: the variables of
b1_mHM_Fluxes_States.nc ("fs_<name>", [interval][cell]) and the Qrouted of
b1_mRM_Fluxes_States.nc ("qrouted", [interval][node]) with the output
settings of its mhm_outputs.nml / mrm_outputs.nml ("out_interval",
"out_flags", "out_interval_mrm", "out_qrouted").
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parents[1]))
from mhm_gb300 import h5read as h5lite  # noqa: E402

if len(sys.argv) < 2:
    sys.exit(f"usage: python {Path(__file__).name} <path of the mHM source tree>")
REF = Path(sys.argv[1])
TD = REF / "test_domain" / "input"
CASE = REF / "check" / "case_00"

# case_00 mhm.nml: &nightdayratio, &panevapo
FNIGHT_PET = [0.1] * 12
FNIGHT_PREC = [0.46, 0.5, 0.52, 0.51, 0.48, 0.5, 0.49, 0.48, 0.52, 0.56, 0.5, 0.47]
FNIGHT_TEMP = [-0.76, -1.3, -1.88, -2.38, -2.72, -2.75, -2.74, -3.04, -2.44, -1.6, -0.94, -0.53]
EVAP_COEFF = [1.3, 1.2, 0.72, 0.75, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.5]
FILE_START = (1989, 1, 1)     # meteo time axis: days since 1989-01-01
SIM_START = (1990, 1, 1)      # eval_Per start 1990-07-01 minus warming_days 181
SIM_DAYS = 546                # .. 1991-06-30
FORCING_DAYS = 730            # forcing rows kept: 1990-01-01 .. 1991-12-31 (case_07 runs both years)
WARMING_DAYS = 181
SCENE2_FROM_DAY = 365         # land-cover scene 1991 from 1991-01-01 on


def output_settings(cdir):
    """timeStep_model_outputs, outputFlxState(1..21), timeStep_model_outputs_mrm
    and outputFlxState_mrm(1) from a case's output namelists."""
    def strip(path):
        return "\n".join(ln.split("!")[0] for ln in path.read_text().splitlines())
    mhm = strip(cdir / "mhm_outputs.nml")
    mrm = strip(cdir / "mrm_outputs.nml") if (cdir / "mrm_outputs.nml").exists() else ""
    interval = int(re.search(r"timeStep_model_outputs\s*=\s*(-?\d+)", mhm).group(1))
    flags = np.zeros(21, np.int32)
    for i, v in re.findall(r"outputFlxState\((\d+)\)\s*=\s*\.(TRUE|FALSE)\.", mhm, re.I):
        flags[int(i) - 1] = v.upper() == "TRUE"
    m = re.search(r"timeStep_model_outputs_mrm\s*=\s*(-?\d+)", mrm)
    interval_mrm = int(m.group(1)) if m else 0
    q = re.search(r"outputFlxState_mrm\(1\)\s*=\s*\.(TRUE|FALSE)\.", mrm, re.I)
    return interval, flags, interval_mrm, int(bool(q and q.group(1).upper() == "TRUE"))


def output_golds(cdir, mask):
    """Aggregated outputs written by a case, packed over the L1 (= L11) mask."""
    interval, flags, interval_mrm, qrouted = output_settings(cdir)
    gold = dict(out_interval=interval, out_flags=flags, out_interval_mrm=interval_mrm, out_qrouted=qrouted)
    fpath = cdir / "output_save" / "b1_mHM_Fluxes_States.nc"
    if fpath.exists():
        f = h5lite.H5File(str(fpath))
        skip = {"easting", "northing", "easting_bnds", "northing_bnds", "lon", "lat", "time", "time_bnds", "bnds"}
        for name in f.group():
            if name not in skip:
                a = f.read(name)
                gold["fs_" + name] = np.stack([a[i][mask] for i in range(a.shape[0])])
        gold["fs_time_bnds"] = f.read("time_bnds")
    rpath = cdir / "output_save" / "b1_mRM_Fluxes_States.nc"
    if rpath.exists():
        f = h5lite.H5File(str(rpath))
        a = f.read("Qrouted")
        gold["qrouted"] = np.stack([a[i][mask] for i in range(a.shape[0])])
        gold["qrouted_time_bnds"] = f.read("time_bnds")
    return gold


def julday(y, m, d):
    a = (14 - m) // 12
    yy, mm = y + 4800 - a, m + 12 * a - 3
    return d + (153 * mm + 2) // 5 + 365 * yy + yy // 4 - yy // 100 + yy // 400 - 32045


def main():
    mrm = h5lite.H5File(str(CASE / "output_save" / "b1_mRM_restart_001.nc"))
    mhm = h5lite.H5File(str(CASE / "output_save" / "b1_mHM_restart_001.nc"))
    mask1 = mrm.read("L1_domain_mask").astype(bool)          # [y][x], north first
    mask11 = mrm.read("L11_domain_mask").astype(bool)
    assert np.array_equal(mask1, mask11)
    n = int(mask1.sum())
    off = julday(*SIM_START) - julday(*FILE_START)
    met = {}
    for key, rel in (("pre", "pre/pre.nc"), ("temp", "tavg/tavg.nc"), ("pet", "pet/pet.nc")):
        f = h5lite.H5File(str(TD / "meteo" / rel))
        a = f.read({"temp": "tavg"}.get(key, key))
        t = f.read("time")
        assert t[off] == off and a.shape[1:] == mask1.shape
        met[key] = np.ascontiguousarray(a[off:off + FORCING_DAYS][:, mask1])
    # daily net radiation (Priestley-Taylor PET): days since 1984-01-02, row 1826 = 1989-01-01
    f = h5lite.H5File(str(TD / "meteo" / "net_rad.nc"))
    a, t = f.read("net_rad"), f.read("time")
    o = int(np.nonzero(t == julday(*SIM_START) - julday(1984, 1, 2))[0][0])
    met["netrad"] = np.ascontiguousarray(a[o:o + FORCING_DAYS][:, mask1])
    # daily absolute vapour pressure and wind speed (Penman-Monteith PET), each on its own time axis
    for key, base in (("eabs", (1983, 12, 31)), ("windspeed", (1984, 1, 1))):
        f = h5lite.H5File(str(TD / "meteo" / f"{key}.nc"))
        a, t = f.read(key), f.read("time")
        o = int(np.nonzero(t == julday(*SIM_START) - julday(*base))[0][0])
        met[key] = np.ascontiguousarray(a[o:o + FORCING_DAYS][:, mask1])
    # daily minimum / maximum temperature (Hargreaves-Samani PET): days since 1933-12-31
    for key in ("tmin", "tmax"):
        f = h5lite.H5File(str(TD / "meteo" / f"{key}.nc"))
        a, t = f.read(key), f.read("time")
        o = int(np.nonzero(t == julday(*SIM_START) - julday(1933, 12, 31))[0][0])
        met[key] = np.ascontiguousarray(a[o:o + FORCING_DAYS][:, mask1])
    n_links = int(mrm.read("L11_fromN").size) - 1
    ffp = mrm.read("L11_nLinkFracFPimp")                      # [scene][y][x], link i at packed position i
    q = np.loadtxt(CASE / "output_save" / "b1_daily_discharge.out", skiprows=1)
    qtext = (CASE / "output_save" / "b1_daily_discharge.out").read_text()
    gold_states = {}
    for name in ("L1_Inter", "L1_snowPack", "L1_sealSTW", "L1_unsatSTW", "L1_satSTW"):
        gold_states[name] = mhm.read(name)[mask1]
    sm = mhm.read("L1_soilMoist")                             # [horizon][y][x]
    gold_states["L1_soilMoist"] = np.stack([sm[h][mask1] for h in range(sm.shape[0])])
    for name in ("L11_qOUT", "L11_Qmod", "L11_C1", "L11_C2"):
        gold_states[name] = mrm.read(name)[mask11]
    for name in ("L11_qTIN", "L11_qTR"):                      # [IT][y][x]
        a = mrm.read(name)
        gold_states[name] = np.stack([a[i][mask11] for i in range(a.shape[0])])
    np.savez_compressed(
        HERE / "case00_run.npz",
        pre=met["pre"], temp=met["temp"], pet=met["pet"], tmin=met["tmin"], tmax=met["tmax"], netrad=met["netrad"],
        eabs=met["eabs"], windspeed=met["windspeed"],
        jul_start=julday(*SIM_START), sim_days=SIM_DAYS,
        warming_days=WARMING_DAYS, scene2_from_day=SCENE2_FROM_DAY,
        from_n=mrm.read("L11_fromN").astype(np.int32), to_n=mrm.read("L11_toN").astype(np.int32),
        mask11=mask11.astype(np.uint8), l11_fdir=mrm.read("L11_fDir")[mask11].astype(np.int32),
        net_perm=mrm.read("L11_netPerm").astype(np.int32), r_order=mrm.read("L11_rOrder").astype(np.int32),
        length=mrm.read("L11_length")[:n_links], slope=mrm.read("L11_slope")[:n_links],
        ffp_imp=np.stack([ffp[s][mask11][:n_links] for s in range(ffp.shape[0])]),
        gauge_node=mrm.read("gaugeNodeList").astype(np.int32),
        l1_l11_id=mrm.read("L1_L11_Id")[mask1].astype(np.int32),
        l11_l1_id=mrm.read("L11_L1_Id")[mask11].astype(np.int32),
        l1_area_km2=mrm.read("L1_domain_cellarea")[mask1], l11_area_km2=mrm.read("L11_domain_cellarea")[mask11],
        latitude=mrm.read("L1_domain_lat")[mask1],
        gold_restart_vars=np.array(sorted(mhm.group())),
        evap_coeff=np.array(EVAP_COEFF), fnight_pet=np.array(FNIGHT_PET), fnight_prec=np.array(FNIGHT_PREC),
        fnight_temp=np.array(FNIGHT_TEMP), gold_q_daily=q[:, 5], gold_q_dmy=q[:, 1:4].astype(np.int32),
        gold_q_obs=q[:, 4], gold_gauge_id=int(qtext.split()[4][5:]),
        gold_daily_text=np.frombuffer(qtext.encode(), np.uint8),
        **{"gold_" + k: v for k, v in gold_states.items()}, **output_golds(CASE, mask1))
    print("wrote", HERE / "case00_run.npz", "cells", n, "links", n_links, "days", SIM_DAYS)


# ---- further check cases on the same inputs (only processCase differs) ----
import make_case00_mpr as mpr_fix  # noqa: E402

# processCase(3), processCase(5), processCase(8)
CASES = {"case_10": (3, -1, 1), "case_12": (4, -1, 1), "case_09": (1, 1, 2), "case_02": (2, 2, 0),
         "case_03": (1, 3, 1), "case_07": (1, 0, 1)}
# cases whose run period differs from case_00's: (simulated days from 1990-01-01, warming days)
PERIODS = {"case_07": (730, 0)}
PARAM_NAMES = ("fSealed", "alpha", "degDayInc", "degDayMax", "degDayNoPre", "fAsp", "karstLoss", "kfastFlow",
               "kSlowFlow", "kBaseFlow", "kPerco", "tempThresh", "unsatThresh", "sealedThresh", "maxInter",
               "fRoots", "soilMoistSat", "soilMoistFC", "wiltingPoint", "soilMoistExp", "petLAIcorFactor",
               "jarvis_thresh_c1", "PrieTayAlpha")


def case_golds(case: str, proc_sm: int, proc_pet: int, proc_rout: int):
    cdir = REF / "check" / case
    mrm = h5lite.H5File(str(cdir / "output_save" / "b1_mRM_restart_001.nc")) if proc_rout else None
    # an optimisation run (case_03) writes no mHM restart
    mfile = cdir / "output_save" / "b1_mHM_restart_001.nc"
    mhm = h5lite.H5File(str(mfile)) if mfile.exists() else None
    mask1 = (mhm or mrm).read("L1_domain_mask").astype(bool)
    names = list(mhm.group()) if mhm else []
    gold = {}
    for name in PARAM_NAMES:
        if "L1_" + name not in names:
            continue
        a = mhm.read("L1_" + name)
        if a.ndim == 2:
            gold["p_" + name] = a[mask1][None]
        else:   # leading dims: [scene][(horizon|month)] then the grid
            lead = a.shape[:-2]
            gold["p_" + name] = a.reshape(-1, *a.shape[-2:])[:, mask1].reshape(*lead, -1)
    for name in ("L1_Inter", "L1_snowPack", "L1_sealSTW", "L1_unsatSTW", "L1_satSTW") if mhm else ():
        gold["s_" + name] = mhm.read(name)[mask1]
    if mhm:
        sm = mhm.read("L1_soilMoist")
        gold["s_L1_soilMoist"] = np.stack([sm[h][mask1] for h in range(sm.shape[0])])
    for name in ("L11_qOUT", "L11_Qmod", "L11_C1", "L11_C2") if mrm else ():
        gold["s_" + name] = mrm.read(name)[mask1]
    q = np.loadtxt(cdir / "output_save" / "b1_daily_discharge.out", skiprows=1) if mrm else np.zeros((0, 6))
    blocks = ["interception1", "snow1", f"soilmoisture{proc_sm}", "directRunoff1",
              {-1: "PETminus1", 0: "PET0", 1: "PET1", 2: "PET2", 3: "PET3"}[proc_pet], "interflow1",
              "percolation1"]
    blocks += [f"routing{proc_rout}"] if proc_rout else []
    blocks += ["geoparameter"]
    gamma = mpr_fix.namelist_values(cdir / "mhm_parameter.nml", blocks)
    dds = cdir / "output_save" / "dds_results.out"
    if dds.exists():
        # an optimisation: the outputs are those of the last evaluation, which is the
        # best one when the last DDS line improved (its 17 digits give the doubles exactly)
        rows = [ln.split() for ln in dds.read_text().splitlines() if ln.strip() and not ln.lstrip().startswith("#")]
        rows = [r for r in rows if len(r) == len(gamma) + 2]
        assert float(rows[-1][1]) < float(rows[-2][1]), "the last evaluation is not the best"
        gamma = [float(x) for x in rows[-1][2:]]
    extra = {}
    if proc_rout == 2:
        # link lengths as mRM sets them up for adaptive routing (cut at their 40th
        # percentile, src/mRM/mo_mrm_net_startup.f90:1441-1447) and the routing step
        n_links = int(mrm.read("L11_fromN").size) - 1
        extra = dict(length=mrm.read("L11_length")[:n_links], ts_rout=float(mrm.read("L11_TSrout")[0]))
    np.savez_compressed(HERE / f"{case.replace('_', '')}_gold.npz", gamma=np.array(gamma), proc_sm=proc_sm,
                        proc_pet=proc_pet, proc_rout=proc_rout, q_daily=q[:, 5], **gold, **extra,
                        restart_vars=np.array(sorted(names)),
                        **({"sim_days": PERIODS[case][0], "warming_days": PERIODS[case][1]} if case in PERIODS else {}),
                        **output_golds(cdir, mask1))
    print("wrote", HERE / f"{case.replace('_', '')}_gold.npz", len(gamma), sorted(gold))


if __name__ == "__main__":
    main()
    for c, procs in CASES.items():
        case_golds(c, *procs)
