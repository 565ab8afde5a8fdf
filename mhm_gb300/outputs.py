"""Names and layout of the aggregated flux/state outputs.

The reference writes the variables selected by outputFlxState(1..21)
(mhm_outputs.nml) to <domain>_mHM_Fluxes_States.nc in a fixed order
(mHM_OutputDataset, src/mHM/mo_write_fluxes_states.f90:82-262), one variable
per soil horizon for the per-horizon quantities.  The device writes its
planes in that same order; this module names them.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

# outputFlxState index -> (variable name, one per horizon, written as interval mean)
VARIABLES = {
    1: ("interception", False, True),
    2: ("snowpack", False, True),
    3: ("SWC_L", True, True),
    4: ("SM_L", True, True),
    5: ("SM_Lall", False, True),
    6: ("sealedSTW", False, True),
    7: ("unsatSTW", False, True),
    8: ("satSTW", False, True),
    18: ("neutrons", False, True),
    9: ("PET", False, False),
    10: ("aET", False, False),
    11: ("Q", False, False),
    12: ("QD", False, False),
    13: ("QIf", False, False),
    14: ("QIs", False, False),
    15: ("QB", False, False),
    16: ("recharge", False, False),
    17: ("soil_infil_L", True, False),
    19: ("aET_L", True, False),
    20: ("preEffect", False, False),
    21: ("Qsm", False, False),
}
# file order of the variables (the dict's insertion order)
ORDER = tuple(VARIABLES)


def flags_from(selected: Sequence[int | str]) -> list[int]:
    """outputFlxState(1..21) as 21 ints from indexes or variable names."""
    by_name = {v[0]: i for i, v in VARIABLES.items()}
    flags = [0] * 21
    for s in selected:
        i = by_name[s] if isinstance(s, str) else int(s)
        flags[i - 1] = 1
    return flags


def plane_names(flags: Sequence[int], n_horizons: int) -> list[str]:
    """Variable name of each output plane, e.g. SWC_L01, SWC_L02, Q."""
    names = []
    for i in ORDER:
        if not flags[i - 1]:
            continue
        name, per_h, _ = VARIABLES[i]
        names.extend([f"{name}{h + 1:02d}" for h in range(n_horizons)] if per_h else [name])
    return names


def daily_discharge(q_steps, warming_days: int, steps_per_day: int):
    """Daily mean discharge of the evaluation period from per-step gauge
    discharge [..., step]: sum(Q(iS:iE)) / nTstepDay over each day after the
    warm-up, summed in step order (mrm_write, src/mRM/mo_mrm_write.f90:138-149)."""
    import numpy as np
    q = np.asarray(q_steps, np.float64)
    days = q[..., warming_days * steps_per_day:]
    days = days.reshape(*days.shape[:-1], -1, steps_per_day)
    return np.cumsum(days, axis=-1)[..., -1] / float(steps_per_day)


def _date_of_jdn(j: int) -> tuple[int, int, int]:
    """(day, month, year) of a Julian day number (Gregorian calendar)."""
    f = j + 1401 + (((4 * j + 274277) // 146097) * 3) // 4 - 38
    e = 4 * f + 3
    g = (e % 1461) // 4
    h = 5 * g + 2
    d = (h % 153) // 5 + 1
    m = (h // 153 + 2) % 12 + 1
    y = e // 1461 - 4716 + (12 + 2 - m) // 12
    return d, m, y


def _f15_7(x: float) -> str:
    s = f"{x:15.7f}"
    return "*" * 15 if len(s) > 15 else s   # a Fortran F edit descriptor that overflows prints asterisks


def format_daily_discharge(jul_eval_start: int, gauge_ids, q_obs, q_sim) -> str:
    """The <domain>_daily_discharge.out text: one line per evaluation day with
    its number, date and observed / simulated discharge of every gauge
    (write_daily_obs_sim_discharge, src/mRM/mo_mrm_write.f90:627-643: header
    format (4a8, n(2X, a5, i10.10, 2X, a5, i10.10)), data (4I8, n(2X, f15.7,
    2X, f15.7))).  q_obs / q_sim are [day][gauge]; missing observations are
    the reference's nodata -9999."""
    q_obs = np.asarray(q_obs, np.float64).reshape(len(q_sim), -1)
    q_sim = np.asarray(q_sim, np.float64).reshape(len(q_sim), -1)
    head = "".join(f"{w:>8s}" for w in ("No", "Day", "Mon", "Year"))
    head += "".join(f"  Qobs_{int(g):010d}  Qsim_{int(g):010d}" for g in gauge_ids)
    lines = [head]
    for t in range(q_sim.shape[0]):
        d, m, y = _date_of_jdn(jul_eval_start + t)
        row = f"{t + 1:8d}{d:8d}{m:8d}{y:8d}"
        row += "".join(f"  {_f15_7(o)}  {_f15_7(s)}" for o, s in zip(q_obs[t], q_sim[t]))
        lines.append(row)
    return "\n".join(lines) + "\n"


def write_daily_discharge(path, jul_eval_start: int, gauge_ids, q_obs, q_sim) -> None:
    with open(path, "w") as f:
        f.write(format_daily_discharge(jul_eval_start, gauge_ids, q_obs, q_sim))
