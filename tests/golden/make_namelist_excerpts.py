#!/usr/bin/env python3
"""Write tests/golden/namelist_excerpts.json: the groups of check cases 00,
04 and 05's mhm.nml and the process blocks of case_00's mhm_parameter.nml
that the drop-in's run configuration reads, as text (the input of
tests/test_namelist.py's pins of the namelist reader)."""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
GROUPS = ["mainconfig", "mainconfig_mhm_mrm", "processselection", "soildata", "panevapo", "nightdayratio",
          "lcover", "lcover_mpr", "time_periods", "evaluation_gauges", "inflow_gauges"]
PARAM_BLOCKS = ["interception1", "snow1", "soilmoisture1", "directrunoff1", "pet0", "interflow1", "percolation1",
                "routing1", "geoparameter"]


def groups(text: str, names: list[str]) -> str:
    out = []
    for n in names:
        m = re.search(r"^\s*&" + n + r"\b.*?^\s*/\s*$", text, re.S | re.M | re.I)
        if not m:
            raise SystemExit(f"group &{n} not found")
        out.append(m.group(0).strip())
    return "\n".join(out) + "\n"


def main():
    if len(sys.argv) < 2:
        sys.exit(f"usage: python {Path(__file__).name} <path of the mHM source tree>")
    ref = Path(sys.argv[1]) / "check"
    out = {f"{c}/mhm.nml": groups((ref / c / "mhm.nml").read_text(), GROUPS) for c in ("case_00", "case_04", "case_05")}
    out["case_00/mhm_parameter.nml"] = groups((ref / "case_00" / "mhm_parameter.nml").read_text(), PARAM_BLOCKS)
    (HERE / "namelist_excerpts.json").write_text(json.dumps(out, indent=1))
    print("wrote", HERE / "namelist_excerpts.json")


if __name__ == "__main__":
    main()
