#!/usr/bin/env python3
"""Build tests/golden/case00_net.npz: the level-0 flow data of the
reference's regression case check/case_00 (the test_domain basin at 500 m:
flow directions, flow accumulation and elevation, packed over the L0 mask in
mHM's column-major (x, y) order), from which mRM's start-up derives the L11
network that case_00's b1_mRM_restart_001.nc holds (its L11 flow
directions, links, routing order, link lengths and slopes, and floodplain
sealed fractions are already in case00_run.npz).

Run as `python make_case00_network.py <mHM source tree>`; the fixture is
committed, so tests never read the reference."""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
if len(sys.argv) < 2:
    sys.exit(f"usage: python {Path(__file__).name} <path of the mHM source tree>")
REF = Path(sys.argv[1])
TD = REF / "test_domain" / "input"
RES_L11 = 24000.0   # case_00 mhm.nml resolution_Routing(1)


def ascii_grid(path: Path):
    with open(path) as f:
        hdr = {}
        for _ in range(6):
            k, v = f.readline().split()
            hdr[k.lower()] = float(v)
        a = np.loadtxt(f)
    return hdr, a


def main():
    hdr, dem = ascii_grid(TD / "morph" / "dem.asc")
    mask2 = dem != hdr["nodata_value"]                  # [y][x], y north first
    out = {}
    for key, rel in (("fdir0", "morph/fdir.asc"), ("facc0", "morph/facc.asc")):
        h, a = ascii_grid(TD / rel)
        assert a.shape == dem.shape and np.array_equal(a != h["nodata_value"], mask2), rel
        out[key] = a[mask2].astype(np.int32)            # packed column-major over mHM's (x, y)
    out["elev0"] = dem[mask2]
    ny, nx = dem.shape
    np.savez_compressed(HERE / "case00_net.npz", nrows0=nx, ncols0=ny, cellsize0=hdr["cellsize"],
                        factor11=int(round(RES_L11 / hdr["cellsize"])), **out)
    print("wrote", HERE / "case00_net.npz", "L0 cells", int(mask2.sum()))


if __name__ == "__main__":
    main()
