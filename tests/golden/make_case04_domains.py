#!/usr/bin/env python3
"""Build tests/golden/case04_gold.npz from the reference's regression case
check/case_04: six domains with their own periods, warm-up lengths and
resolutions.  The four on the test_domain inputs are kept:

  domain 1: L1 = L11 = 24 km, 1990-01-02 .. 1990-12-31 (180 warm-up days)
  domain 2: L1 = 12 km, L11 = 24 km (four L1 cells per L11 node where the
            mask is full), 1990-07-05 .. 1992-12-31, land-cover scene switch
            on 1991-01-01
  domain 4: L1 = L11 = 24 km, 1989-07-06 .. 1990-12-31 (360 warm-up days)
  domain 5: L1 = L11 = 12 km, 1991-11-12 .. 1992-12-31 (50 warm-up days)

(domains 3 and 6 read test_domain_2, whose temperature and PET files are not
in the reference tree).  Per domain: the daily forcing of the run on the
domain's L1 cells (the 24 km meteo grid; a 12 km L1 cell takes the value of
the 24 km cell it lies in), the network mRM built and the L1 -> L11 mapping
(b<d>_mRM_restart_00<d>.nc), the effective L1 parameters and final states
(b<d>_mHM_restart_00<d>.nc) and the daily discharge file.  Cell arrays are
packed in the row-major order of the north-first grids, as for case_00."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from mhm_gb300 import h5read as h5lite  # noqa: E402

if len(sys.argv) < 2:
    sys.exit(f"usage: python {Path(__file__).name} <path of the mHM source tree>")
REF = Path(sys.argv[1])
CASE = REF / "check" / "case_04"
TD = REF / "test_domain" / "input"
FILE_START = (1989, 1, 1)          # meteo time axis: days since 1989-01-01
# domain -> (evaluation start, evaluation end, warming days)   (&time_periods of case_04's mhm.nml)
DOMAINS = {1: ((1990, 7, 1), (1990, 12, 31), 180), 2: ((1991, 1, 1), (1992, 12, 31), 180),
           4: ((1990, 7, 1), (1990, 12, 31), 360), 5: ((1992, 1, 1), (1992, 12, 31), 50)}
SCENE2_FROM = (1991, 1, 1)         # lc_1991 from 1991 on (lcoveryearstart(2) = 1991)
PARAMS = ("fSealed", "alpha", "degDayInc", "degDayMax", "degDayNoPre", "fAsp", "karstLoss", "kfastFlow",
          "kSlowFlow", "kBaseFlow", "kPerco", "tempThresh", "unsatThresh", "sealedThresh", "maxInter",
          "fRoots", "soilMoistSat", "soilMoistFC", "wiltingPoint", "soilMoistExp")


def julday(y, m, d):
    a = (14 - m) // 12
    yy, mm = y + 4800 - a, m + 12 * a - 3
    return d + (153 * mm + 2) // 5 + 365 * yy + yy // 4 - yy // 100 + yy // 400 - 32045


def main():
    met24 = {}
    for key, rel in (("pre", "pre/pre.nc"), ("temp", "tavg/tavg.nc"), ("pet", "pet/pet.nc")):
        f = h5lite.H5File(str(TD / "meteo" / rel))
        met24[key] = f.read({"temp": "tavg"}.get(key, key))
        assert f.read("time")[0] == 0
    out = {}
    for d, (e0, e1, warm) in DOMAINS.items():
        mrm = h5lite.H5File(str(CASE / "output_save" / f"b{d}_mRM_restart_00{d}.nc"))
        mhm = h5lite.H5File(str(CASE / "output_save" / f"b{d}_mHM_restart_00{d}.nc"))
        mask1 = mhm.read("L1_domain_mask").astype(bool)
        mask11 = mrm.read("L11_domain_mask").astype(bool)
        start = julday(*e0) - warm
        n_days = julday(*e1) - start + 1
        off = start - julday(*FILE_START)
        f = mask1.shape[0] // met24["pre"].shape[1]          # L1 cells per meteo cell along an axis
        assert mask1.shape == (met24["pre"].shape[1] * f, met24["pre"].shape[2] * f)
        yy, xx = np.nonzero(mask1)
        pre = f"d{d}_"
        for key, a in met24.items():
            out[pre + key] = np.ascontiguousarray(a[off:off + n_days][:, yy // f, xx // f])
        n_links = int(mrm.read("L11_fromN").size) - 1
        ffp = mrm.read("L11_nLinkFracFPimp")
        out.update({
            pre + "jul_start": start, pre + "sim_days": n_days, pre + "warming_days": warm,
            pre + "scene0": int(start >= julday(*SCENE2_FROM)),
            pre + "scene2_from_day": max(0, julday(*SCENE2_FROM) - start) if start < julday(*SCENE2_FROM) <= start + n_days - 1 else -1,
            pre + "from_n": mrm.read("L11_fromN").astype(np.int32), pre + "to_n": mrm.read("L11_toN").astype(np.int32),
            pre + "net_perm": mrm.read("L11_netPerm").astype(np.int32),
            pre + "length": mrm.read("L11_length")[:n_links], pre + "slope": mrm.read("L11_slope")[:n_links],
            pre + "ffp_imp": np.stack([ffp[s][mask11][:n_links] for s in range(ffp.shape[0])]),
            pre + "gauge_node": mrm.read("gaugeNodeList").astype(np.int32),
            pre + "l1_l11_id": mrm.read("L1_L11_Id")[mask1].astype(np.int32),
            pre + "l11_l1_id": mrm.read("L11_L1_Id")[mask11].astype(np.int32),
            pre + "l1_area_km2": mrm.read("L1_domain_cellarea")[mask1],
            pre + "l11_area_km2": mrm.read("L11_domain_cellarea")[mask11],
            pre + "latitude": mrm.read("L1_domain_lat")[mask1],
        })
        for name in PARAMS:
            a = mhm.read("L1_" + name)
            lead = a.shape[:-2]
            out[pre + "p_" + name] = a.reshape(-1, *a.shape[-2:])[:, mask1].reshape(*lead, -1)
        for name in ("L1_Inter", "L1_snowPack", "L1_sealSTW", "L1_unsatSTW", "L1_satSTW"):
            out[pre + "s_" + name] = mhm.read(name)[mask1]
        sm = mhm.read("L1_soilMoist")
        out[pre + "s_L1_soilMoist"] = np.stack([sm[h][mask1] for h in range(sm.shape[0])])
        for name in ("L11_qOUT", "L11_Qmod", "L11_C1", "L11_C2"):
            out[pre + "s_" + name] = mrm.read(name)[mask11]
        path = CASE / "output_save" / f"b{d}_daily_discharge.out"
        text = path.read_text()
        q = np.loadtxt(path, skiprows=1)
        out[pre + "gauge_ids"] = np.array([int(w[5:]) for w in text.split()[4:6:2]], np.int32)
        out[pre + "q_obs"] = q[:, 4::2]
        out[pre + "q_sim"] = q[:, 5::2]
        out[pre + "text"] = np.frombuffer(text.encode(), np.uint8)
        print("domain", d, "L1", int(mask1.sum()), "L11", int(mask11.sum()), "days", n_days, "eval", q.shape[0])
    np.savez_compressed(HERE / "case04_gold.npz", **out)
    print("wrote", HERE / "case04_gold.npz")


if __name__ == "__main__":
    main()
