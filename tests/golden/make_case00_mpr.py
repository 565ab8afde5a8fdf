#!/usr/bin/env python3
"""Build tests/golden/case00_mpr.npz: the parameter-regionalisation inputs of
the reference's regression case check/case_00 (the test_domain basin) and the
L1 effective parameters the reference itself wrote for it
(check/case_00/output_save/b1_mHM_restart_001.nc).

Run as `python make_case00_mpr.py <mHM source tree>` (the tree is REF); the
fixture is committed, so tests never read the reference.  What is restated
here (input handling, not the hot path):
  * ESRI ASCII grids -> mHM's (x, y) grids packed column-major over the L0
    mask (src/common/mo_read_spatial_data.f90:94-204 reads rows north first
    and transposes), i.e. row-major order of the ASCII rows;
  * read_soil_LUT, iFlag_soilDB = 0 (src/MPR/mo_soil_database.f90:66-280):
    horizons cut at the tillage depth, clay/sand clamped at 1 % and rescaled
    when they exceed 100 % (the reference rescales sand with the already
    rescaled clay), RZdepth = deepest lower boundary;
  * the LAI and geology class tables;
  * read_data's corrections of the L0 inputs (src/MPR/mo_read_wrapper.f90:
    282-283, 335-336): slope >= 0.01, aspect >= 1, LAI within [1e-10, 30];
  * init_lowres_level (src/common/mo_grid.f90:58-183): L1 blocks of
    resolution_hydrology / L0 cellsize L0 cells;
  * the `value` column of case_00's mhm_parameter.nml for the process cases
    of its mhm.nml (processCase = 1,1,1,1,0,1,1,1,1,0).
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

TILLAGE = 200.0          # case_00 mhm.nml tillageDepth
HORIZON_DEPTH = [200.0, 0.0]  # soil_depth(1) = 200; the last entry becomes RZdepth
RES_L1 = 24000.0         # resolution_hydrology(1)
FRAC_SEALED_CITY = 0.6   # fracSealed_cityArea


def ascii_grid(path: Path):
    with open(path) as f:
        hdr = {}
        for _ in range(6):
            k, v = f.readline().split()
            hdr[k.lower()] = float(v)
        a = np.loadtxt(f)
    return hdr, a


def soil_lut(path: Path):
    rows = []
    with open(path) as f:
        n_types = int(f.readline().split()[1])
        f.readline()
        for line in f:
            p = line.split()
            if len(p) >= 7:
                rows.append([float(x) for x in p[:7]])
    rows = np.array(rows)
    ids = rows[:, 0].astype(int)
    n_hor = np.zeros(n_types + 1, int)
    rz = np.full(n_types + 1, -9999.0)
    n_till = np.full(n_types + 1, -9999, int)
    for ii, jj, up, down, *_ in rows:
        ii, jj = int(ii), int(jj)
        n_hor[ii] = jj
        rz[ii] = max(rz[ii], np.round(down))
    for ii, jj, up, down, *_ in rows:  # a horizon cut by the tillage depth adds one
        ii, jj = int(ii), int(jj)
        if TILLAGE > np.round(up) and TILLAGE < np.round(down):
            n_hor[ii] += 1
        if TILLAGE > np.round(up) and TILLAGE <= np.round(down):
            n_till[ii] = jj
    mh = n_hor.max()
    UD = np.full((n_types + 1, mh), -9999.0)
    LD = UD.copy()
    clay = UD.copy()
    sand = UD.copy()
    dbm = UD.copy()
    kk = 0
    for ii, jj, up, down, cly, snd, bd in rows:
        jj, nH = int(ii), int(jj)
        if cly < 1.0:
            cly = 1.0
        if snd < 1.0:
            snd = 1.0
        if cly + snd > 100.0:
            cly = cly / (cly + snd)
            snd = snd / (cly + snd)
        if TILLAGE > np.round(up) and TILLAGE < np.round(down):
            UD[jj, nH - 1] = np.round(up)
            LD[jj, nH - 1] = TILLAGE
            clay[jj, nH - 1], sand[jj, nH - 1], dbm[jj, nH - 1] = cly, snd, bd
            up = TILLAGE
            kk = 1
        if kk == 1:
            nH += 1
        UD[jj, nH - 1] = np.round(up)
        LD[jj, nH - 1] = np.round(down)
        clay[jj, nH - 1], sand[jj, nH - 1], dbm[jj, nH - 1] = cly, snd, bd
        if nH == n_hor[jj]:
            kk = 0
    assert len(set(ids)) == n_types
    s = slice(1, None)
    return (n_hor[s].astype(np.int32), n_till[s].astype(np.int32), UD[s], LD[s], sand[s], clay[s], dbm[s], rz[s])


def lai_lut(path: Path):
    with open(path) as f:
        n = int(f.readline().split()[1])
        f.readline()
        tab = np.zeros((n, 12))
        ids = []
        for i in range(n):
            p = f.readline().split()
            ids.append(int(p[0]))
            tab[i] = [float(x) for x in p[2:14]]
    assert ids == list(range(1, n + 1))
    return tab


def geology(path: Path):
    with open(path) as f:
        n = int(f.readline().split()[1])
        f.readline()
        units, kar = [], []
        for _ in range(n):
            p = f.readline().split()
            units.append(int(p[1]))
            kar.append(int(p[2]))
    return np.array(units, np.int32), np.array(kar, np.int32)


def namelist_values(path: Path, blocks: list[str]) -> list[float]:
    """`value` column (third number) of the named namelist blocks, in order."""
    text = path.read_text()
    out = []
    for b in blocks:
        m = re.search(r"&" + re.escape(b) + r"\b(.*?)\n\s*/", text, re.S | re.I)
        if not m:
            raise ValueError(f"block {b} not found")
        for line in m.group(1).splitlines():
            line = line.split("!")[0]
            if "=" not in line:
                continue
            nums = [float(x) for x in line.split("=", 1)[1].replace(",", " ").split()]
            out.append(nums[2])
    return out


def main():
    hdr, dem = ascii_grid(TD / "morph" / "dem.asc")
    mask2 = dem != hdr["nodata_value"]                  # [y][x], y north first
    maps = {}
    for key, rel in (("soil", "morph/soil_class.asc"), ("lai", "morph/LAI_class.asc"),
                     ("geo", "morph/geology_class.asc"), ("slope", "morph/slope.asc"),
                     ("aspect", "morph/aspect.asc"), ("lc1981", "luse/lc_1981.asc"),
                     ("lc1991", "luse/lc_1991.asc")):
        h, a = ascii_grid(TD / rel)
        assert a.shape == dem.shape and np.array_equal(a != h["nodata_value"], mask2), rel
        maps[key] = a[mask2]                            # packed column-major over mHM's (x, y)
    # read_data's corrections (src/MPR/mo_read_wrapper.f90:282-283, 335-336)
    maps["slope"] = np.where(maps["slope"] < 0.01, 0.01, maps["slope"])
    maps["aspect"] = np.where(maps["aspect"] < 1.0, 1.0, maps["aspect"])
    f = int(round(RES_L1 / hdr["cellsize"]))
    ny, nx = dem.shape
    nr1, nc1 = -(-nx // f), -(-ny // f)                 # mHM rows = x, cols = y
    mask1 = np.zeros((nc1, nr1), bool)                  # [jc][ic]
    for j in range(ny):
        for i in range(nx):
            if mask2[j, i]:
                mask1[j // f, i // f] = True
    up, down, left, right, nsub = [], [], [], [], []
    for jc in range(nc1):
        for ic in range(nr1):
            if not mask1[jc, ic]:
                continue
            iu, idn = ic * f + 1, min((ic + 1) * f, nx)
            jl, jr = jc * f + 1, min((jc + 1) * f, ny)
            up.append(iu), down.append(idn), left.append(jl), right.append(jr)
            nsub.append(int(mask2[jl - 1:jr, iu - 1:idn].sum()))
    n_hor, n_till, UD, LD, sand, clay, dbm, rz = soil_lut(TD / "morph" / "soil_classdefinition.txt")
    units, kar = geology(TD / "morph" / "geology_classdefinition.txt")
    gamma = namelist_values(CASE / "mhm_parameter.nml",
                            ["interception1", "snow1", "soilmoisture1", "directRunoff1", "PET0", "interflow1",
                             "percolation1", "routing1", "geoparameter"])
    # golden L1 parameters (per land-cover scene), packed over the L1 mask
    h5 = h5lite.H5File(str(CASE / "output_save" / "b1_mHM_restart_001.nc"))
    m1 = h5.read("L1_domain_mask").astype(bool)
    assert m1.shape == mask1.shape and np.array_equal(m1, mask1)
    gold = {}
    for name in ("fSealed", "alpha", "degDayInc", "degDayMax", "degDayNoPre", "fAsp", "karstLoss", "kfastFlow",
                 "kSlowFlow", "kBaseFlow", "kPerco", "tempThresh", "unsatThresh", "sealedThresh", "maxInter",
                 "fRoots", "soilMoistSat", "soilMoistFC", "wiltingPoint", "soilMoistExp"):
        a = h5.read("L1_" + name)
        gold[name] = np.stack([a[s][..., m1] if a.ndim > 2 else a[m1] for s in range(a.shape[0])]) \
            if a.ndim >= 3 else a[m1][None]
    np.savez_compressed(
        HERE / "case00_mpr.npz",
        nrows0=nx, ncols0=ny, factor=f, mask0=np.packbits(mask2.reshape(-1)), n_mask0=mask2.size,
        l1_up=np.array(up, np.int32), l1_down=np.array(down, np.int32), l1_left=np.array(left, np.int32),
        l1_right=np.array(right, np.int32), l1_nsub=np.array(nsub, np.int32),
        soil_id0=maps["soil"].astype(np.int16), lai_class0=maps["lai"].astype(np.int8),
        geo_unit0=maps["geo"].astype(np.int8), slope0=maps["slope"], aspect0=maps["aspect"], lcover0=np.stack([maps["lc1981"], maps["lc1991"]]).astype(np.int8),
        soil_n_hor=n_hor, soil_n_till=n_till, soil_ud=UD, soil_ld=LD, soil_sand=sand, soil_clay=clay,
        soil_dbm=dbm, soil_rz_depth=rz,
        lai_lut=np.clip(lai_lut(TD / "morph" / "LAI_classdefinition.txt"), 1.0e-10, 30.0),
        geo_unit_list=units, geo_unit_kar=kar, gamma=np.array(gamma), horizon_depth=np.array(HORIZON_DEPTH),
        frac_sealed_city=FRAC_SEALED_CITY, **{"gold_" + k: v for k, v in gold.items()})
    print("wrote", HERE / "case00_mpr.npz", "L1 cells", len(up), "L0 cells", int(mask2.sum()),
          "gamma", len(gamma))


if __name__ == "__main__":
    main()
