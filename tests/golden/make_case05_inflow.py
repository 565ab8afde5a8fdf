#!/usr/bin/env python3
"""Build tests/golden/case05_gold.npz from the reference's regression case
check/case_05: three domains on the test_domain inputs of case_00 (same
parameters, processes, periods and network), each evaluated at gauges 398 and
333, with gauge 333 also an inflow gauge -- not a headwater in domain 1,
a headwater in domain 2, absent in domain 3.

Written per domain d (1..3): the daily simulated and observed discharge of
both gauges (b<d>_daily_discharge.out, and its text), the gauge and inflow
gauge node lists, the effective L1 parameters and the final states of
b<d>_mHM_restart_00<d>.nc / b<d>_mRM_restart_00<d>.nc; and once: the inflow gauge's daily discharge
(test_domain/input/gauge/00333.txt) from 1990-01-01 on."""
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
CASE = REF / "check" / "case_05"
SIM_START = (1990, 1, 1)
FORCING_DAYS = 730
HEADWATER = {1: 0, 2: 1}     # &inflow_gauges inflowgauge_headwater(d, 1) of domains 1 and 2
N_INFLOW = {1: 1, 2: 1, 3: 0}  # noinflowgauges_domain(1:3)
PARAMS = ("fSealed", "alpha", "degDayInc", "degDayMax", "degDayNoPre", "fAsp", "karstLoss", "kfastFlow",
          "kSlowFlow", "kBaseFlow", "kPerco", "tempThresh", "unsatThresh", "sealedThresh", "maxInter",
          "fRoots", "soilMoistSat", "soilMoistFC", "wiltingPoint", "soilMoistExp")


def inflow_series(path: Path, start, n_days: int) -> np.ndarray:
    """Daily values of a gauge file (5 header lines, then 'YYYY MM DD HH MM value')
    from `start` on."""
    rows = [ln.split() for ln in path.read_text().splitlines()[5:] if ln.strip()]
    dates = [tuple(int(x) for x in r[:3]) for r in rows]
    i0 = dates.index(tuple(start))
    q = np.array([float(r[5]) for r in rows[i0:i0 + n_days]])
    assert q.size == n_days and np.all(q >= 0.0)
    return q


def main():
    out = {"inflow_q333": inflow_series(REF / "test_domain" / "input" / "gauge" / "00333.txt", SIM_START,
                                        FORCING_DAYS)}
    for d in (1, 2, 3):
        mrm = h5lite.H5File(str(CASE / "output_save" / f"b{d}_mRM_restart_00{d}.nc"))
        mhm = h5lite.H5File(str(CASE / "output_save" / f"b{d}_mHM_restart_00{d}.nc"))
        mask = mrm.read("L1_domain_mask").astype(bool)
        path = CASE / "output_save" / f"b{d}_daily_discharge.out"
        text = path.read_text()
        q = np.loadtxt(path, skiprows=1)
        ids = [int(w[5:]) for w in text.split()[4:8:2]]
        pre = f"d{d}_"
        out[pre + "gauge_ids"] = np.array(ids, np.int32)
        out[pre + "q_obs"] = q[:, 4::2]
        out[pre + "q_sim"] = q[:, 5::2]
        out[pre + "text"] = np.frombuffer(text.encode(), np.uint8)
        out[pre + "gauge_node"] = mrm.read("gaugeNodeList").astype(np.int32)
        n_in = N_INFLOW[d]
        out[pre + "inflow_node"] = (mrm.read("InflowGaugeNodeList").astype(np.int32).reshape(-1)[:n_in]
                                    if n_in else np.zeros(0, np.int32))
        out[pre + "inflow_headwater"] = np.array([HEADWATER.get(d, 0)] * n_in, np.int32)
        # the effective parameters the time loop used, [scene][(horizon|LAI step)][cell]
        # or [(LAI step)][cell] for the scene-independent ones: case_05 reads a
        # monthly gridded LAI series (timeStep_LAI_input = -2), so maxInter has
        # one entry per month of the run (1990-01 .. 1991-06)
        for name in PARAMS:
            a = mhm.read("L1_" + name)
            lead = a.shape[:-2]
            out[pre + "p_" + name] = a.reshape(-1, *a.shape[-2:])[:, mask].reshape(*lead, -1)
        for name in ("L1_Inter", "L1_snowPack", "L1_sealSTW", "L1_unsatSTW", "L1_satSTW"):
            out[pre + "s_" + name] = mhm.read(name)[mask]
        sm = mhm.read("L1_soilMoist")
        out[pre + "s_L1_soilMoist"] = np.stack([sm[h][mask] for h in range(sm.shape[0])])
        for name in ("L11_qOUT", "L11_Qmod", "L11_C1", "L11_C2"):
            out[pre + "s_" + name] = mrm.read(name)[mask]
        for name in ("L11_qTIN", "L11_qTR"):
            a = mrm.read(name)
            out[pre + "s_" + name] = np.stack([a[i][mask] for i in range(a.shape[0])])
    np.savez_compressed(HERE / "case05_gold.npz", **out)
    print("wrote", HERE / "case05_gold.npz", sorted(out))


if __name__ == "__main__":
    main()
