"""Seeded synthetic basins, effective parameters and forcing.

No public dataset is involved: the generators follow the shapes, sizes and
value distributions of the workloads this package is measured on (hourly
forcing, 3-6 soil horizons, D8 networks draining to one outlet).

Grids follow the reference's conventions: cells are packed column-major over
the mask (src/common/mo_grid.f90:145-150), L11 cells are blocks of
`l11_factor` x `l11_factor` L1 cells (L11_L1_mapping,
src/mRM/mo_mrm_net_startup.f90:61-226), links come from L11 D8 directions in
cell order with sinks dropped (L11_set_network_topology, :630-727) and the
routing order is the reference's (computed by the library's
mhm_routing_order).  Flow-direction codes are mRM's (moveDownOneCell,
:1768-1801: 1 E, 2 SE, 4 S, 8 SW, 16 W, 32 NW, 64 N, 128 NE, 0 sink).
"""
from __future__ import annotations

import ctypes as C
import heapq
from dataclasses import dataclass, field

import numpy as np

# D8: code -> (drow, dcol); row index grows southwards
D8 = {1: (0, 1), 2: (1, 1), 4: (1, 0), 8: (1, -1), 16: (0, -1), 32: (-1, -1), 64: (-1, 0), 128: (-1, 1)}
_NEIGH = [(dr, dc) for dr in (-1, 0, 1) for dc in (-1, 0, 1) if (dr, dc) != (0, 0)]
_CODE = {v: k for k, v in D8.items()}

# 2000-01-01 as a Julian day number (FORCES julday(1, 1, 2000))
JUL_2000 = 2451545


@dataclass
class Domain:
    nrows: int
    ncols: int
    n_horizons: int
    l11_factor: int
    horizon_depth: np.ndarray          # [H] mm, last = root-zone depth
    l1_area_km2: np.ndarray            # [N]
    l1_l11_id: np.ndarray              # [N] int32, 1-based
    nrows11: int
    ncols11: int
    l11_area_km2: np.ndarray           # [L]
    l11_l1_id: np.ndarray              # [L] int32 (unused when map_flag = 1)
    fdir11: np.ndarray                 # [L] int32 mRM codes, packed
    cell_row11: np.ndarray             # [L] 1-based
    cell_col11: np.ndarray             # [L] 1-based
    id11_2d: np.ndarray                # [ncols11, nrows11] (column-major 2-D id grid)
    elev11: np.ndarray                 # [L] filled elevation [m]
    n_outlets: int
    from_n: np.ndarray                 # [L] int32 (valid 1..nLinks)
    to_n: np.ndarray                   # [L]
    net_perm: np.ndarray               # [L]
    r_order: np.ndarray                # [L]
    length: np.ndarray                 # [nLinks] m
    slope: np.ndarray                  # [nLinks]
    ffp_imp: np.ndarray                # [nLinks]
    gauge_node: np.ndarray             # [G] int32, 1-based
    latitude: np.ndarray               # [N] degrees
    timestep: int = 1
    jul_start: int = JUL_2000
    evap_coeff: np.ndarray = field(default_factory=lambda: np.array(
        [1.30, 1.20, 0.72, 0.75, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.00, 1.50]))
    # &nightDayRatio of mhm.nml
    fday_prec: np.ndarray = field(default_factory=lambda: np.full(12, 0.5))
    fnight_prec: np.ndarray = field(default_factory=lambda: np.full(12, 0.5))
    fday_pet: np.ndarray = field(default_factory=lambda: np.full(12, 0.95))
    fnight_pet: np.ndarray = field(default_factory=lambda: np.full(12, 0.05))
    fday_temp: np.ndarray = field(default_factory=lambda: np.full(12, -0.988))
    fnight_temp: np.ndarray = field(default_factory=lambda: np.full(12, 0.988))

    @property
    def n_cells(self) -> int:
        return self.nrows * self.ncols

    @property
    def n_nodes(self) -> int:
        return self.nrows11 * self.ncols11

    @property
    def n_links(self) -> int:
        return self.n_nodes - self.n_outlets

    def depth_stats(self) -> tuple[int, int]:
        """(number of topological levels, widest level) of the L11 network."""
        L = self.n_nodes
        level = np.zeros(L, np.int64)
        for r in range(self.n_links):
            i = self.net_perm[r] - 1
            f, t = self.from_n[i] - 1, self.to_n[i] - 1
            level[t] = max(level[t], level[f] + 1)
        counts = np.bincount(level)
        return int(level.max() + 1), int(counts.max())


def _priority_flood_d8(z: np.ndarray, outlet: tuple[int, int]) -> tuple[np.ndarray, np.ndarray]:
    """D8 directions of a tree draining every cell to `outlet`: priority flood
    (Barnes et al. 2014) seeded at the outlet only, so pits are filled and all
    flow ends there.  Returns (fdir[nr, nc] mRM codes, filled elevation)."""
    nr, nc = z.shape
    fdir = np.zeros((nr, nc), np.int32)
    filled = z.copy()
    seen = np.zeros((nr, nc), bool)
    heap = [(float(z[outlet]), 0, outlet)]
    seen[outlet] = True
    counter = 1
    while heap:
        e, _, (i, j) = heapq.heappop(heap)
        for dr, dc in _NEIGH:
            ii, jj = i + dr, j + dc
            if 0 <= ii < nr and 0 <= jj < nc and not seen[ii, jj]:
                seen[ii, jj] = True
                fdir[ii, jj] = _CODE[(-dr, -dc)]  # from (ii, jj) towards (i, j)
                ne = max(float(z[ii, jj]), e + 1e-3)
                filled[ii, jj] = ne
                heapq.heappush(heap, (ne, counter, (ii, jj)))
                counter += 1
    return fdir, filled


def _fractal_noise(rng: np.random.Generator, nr: int, nc: int, beta: float) -> np.ndarray:
    """Spectral 1/f^beta noise, unit variance."""
    ky = np.fft.fftfreq(nr)[:, None]
    kx = np.fft.rfftfreq(nc)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    amp = k ** (-beta / 2.0)
    amp[0, 0] = 0.0
    spec = (rng.standard_normal((nr, nc // 2 + 1)) + 1j * rng.standard_normal((nr, nc // 2 + 1))) * amp
    f = np.fft.irfft2(spec, s=(nr, nc))
    return f / (f.std() + 1e-30)


def routing_order(from_n: np.ndarray, to_n: np.ndarray, n_nodes: int, n_outlets: int):
    """netPerm, rOrder of the reference's L11_routing_order (via the library)."""
    from . import _lib
    L = _lib.load()
    perm = np.zeros(n_nodes, np.int32)
    rord = np.zeros(n_nodes, np.int32)
    ip = C.POINTER(C.c_int32)
    fn = np.ascontiguousarray(from_n, np.int32)
    tn = np.ascontiguousarray(to_n, np.int32)
    rc = L.mhm_routing_order(n_nodes, n_outlets, fn.ctypes.data_as(ip), tn.ctypes.data_as(ip),
                             perm.ctypes.data_as(ip), rord.ctypes.data_as(ip))
    if rc != 0:
        raise RuntimeError("mhm_routing_order failed")
    return perm, rord


def network_topology(fdir11: np.ndarray, rows: np.ndarray, cols: np.ndarray, id2d: np.ndarray):
    """L11_set_network_topology (src/mRM/mo_mrm_net_startup.f90:630-727)."""
    L = len(fdir11)
    from_n = np.full(L, -9999, np.int32)
    to_n = np.full(L, -9999, np.int32)
    jj = 0
    for kk in range(L):
        ic, jc = int(rows[kk]), int(cols[kk])
        d = D8.get(int(fdir11[kk]))
        if d is not None:
            ic, jc = ic + d[0], jc + d[1]
        tn = int(id2d[jc - 1, ic - 1])
        if kk + 1 == tn:
            continue
        from_n[jj] = kk + 1
        to_n[jj] = tn
        jj += 1
    return from_n, to_n, L - jj


def make_domain(nrows: int = 96, ncols: int = 96, n_horizons: int = 3, l11_factor: int = 4, seed: int = 1,
                cellsize_m: float = 1000.0, dem_kind: str = "plane", fractal_beta: float = 3.0,
                tilt: float = 0.002, lat0: float = 50.0, timestep: int = 1,
                jul_start: int = JUL_2000, ridges: int = 0, order=None) -> Domain:
    """A rectangular basin: L1 grid nrows x ncols, L11 = l11_factor^2 L1 cells,
    DEM (tilted plane + N(0, 5 m), or fractal noise + tilt) draining through
    D8 to one outlet at the lowest corner.  `order(from_n, to_n, n_nodes,
    n_outlets) -> (netPerm, rOrder)` computes the routing order (default: the
    library's mhm_routing_order)."""
    rng = np.random.default_rng(seed)
    N = nrows * ncols
    nr11 = -(-nrows // l11_factor)
    nc11 = -(-ncols // l11_factor)
    L = nr11 * nc11
    H = n_horizons
    # horizon depths: 200, 500, ... mm, the last one to the root-zone depth
    base = [200.0, 500.0, 800.0, 1100.0, 1400.0, 1700.0, 2000.0]
    hd = np.array(base[:H - 1] + [max(2000.0, base[H - 2] + 500.0) if H > 1 else 1000.0], np.float64)
    l1_area = np.full(N, cellsize_m * cellsize_m * 1e-6)
    # L11 ids: column-major over the (full) L11 mask
    id11_2d = np.arange(1, L + 1, dtype=np.int32).reshape(nc11, nr11)  # [col][row]
    ii, jj = np.meshgrid(np.arange(nrows), np.arange(ncols), indexing="ij")  # L1 row/col
    l1_l11 = id11_2d[jj // l11_factor, ii // l11_factor]  # [nrows, ncols]
    l1_l11_id = np.ascontiguousarray(l1_l11.T.reshape(-1), np.int32)  # column-major pack
    rows11 = np.tile(np.arange(1, nr11 + 1, dtype=np.int32), nc11)
    cols11 = np.repeat(np.arange(1, nc11 + 1, dtype=np.int32), nr11)
    cs11 = cellsize_m * l11_factor
    l11_area = np.full(L, cs11 * cs11 * 1e-6)
    # the L1 cell at the block's upper-left corner (used only when map_flag = 0)
    l11_l1_id = np.ascontiguousarray(((cols11 - 1) * l11_factor * nrows + (rows11 - 1) * l11_factor + 1), np.int32)
    # DEM at L11 (row 0 = north); outlet at the south-east corner
    r = np.arange(nr11)[:, None]
    c = np.arange(nc11)[None, :]
    if dem_kind == "fractal":
        z = 50.0 * _fractal_noise(rng, nr11, nc11, fractal_beta) + tilt * cs11 * ((nr11 - 1 - r) + (nc11 - 1 - c))
        # folded main valley: `ridges` east-west ridges, each open at alternating
        # ends, lengthen the trunk river (the knob for the network depth)
        for q in range(ridges):
            rr = (q + 1) * nr11 // (ridges + 1)
            gap = max(2, nc11 // 25)
            cols = slice(gap, nc11) if q % 2 == (ridges % 2) else slice(0, nc11 - gap)
            z[rr, cols] += 1e4
    else:
        z = tilt * cs11 * ((nr11 - 1 - r) + (nc11 - 1 - c)) + rng.normal(0.0, 5.0, (nr11, nc11))
    z = z.astype(np.float64)
    outlet = (nr11 - 1, nc11 - 1)
    z[outlet] = z.min() - 1.0
    fdir2d, filled = _priority_flood_d8(z, outlet)
    fdir11 = np.ascontiguousarray(fdir2d.T.reshape(-1), np.int32)  # column-major pack
    elev11 = filled.T.reshape(-1)
    from_n, to_n, n_out = network_topology(fdir11, rows11, cols11, id11_2d)
    perm, rord = (order or routing_order)(from_n, to_n, L, n_out)
    nl = L - n_out
    diag = np.array([fdir11[from_n[i] - 1] in (2, 8, 32, 128) for i in range(nl)], bool)
    length = cs11 * np.where(diag, np.sqrt(2.0), 1.0) * rng.uniform(1.0, 1.3, nl)
    drop = elev11[from_n[:nl] - 1] - elev11[to_n[:nl] - 1]
    slope = np.maximum(1e-4, drop / length)
    ffp = rng.uniform(0.0, 0.1, nl)
    outlet_id = int(id11_2d[outlet[1], outlet[0]])
    lat = lat0 + (nrows - 1 - ii.T.reshape(-1)) * cellsize_m / 111_000.0
    return Domain(nrows=nrows, ncols=ncols, n_horizons=H, l11_factor=l11_factor, horizon_depth=hd,
                  l1_area_km2=l1_area, l1_l11_id=l1_l11_id, nrows11=nr11, ncols11=nc11,
                  l11_area_km2=l11_area, l11_l1_id=l11_l1_id, fdir11=fdir11, cell_row11=rows11,
                  cell_col11=cols11, id11_2d=id11_2d, elev11=elev11, n_outlets=n_out,
                  from_n=from_n, to_n=to_n, net_perm=perm, r_order=rord,
                  length=np.ascontiguousarray(length), slope=np.ascontiguousarray(slope),
                  ffp_imp=np.ascontiguousarray(ffp), gauge_node=np.array([outlet_id], np.int32),
                  latitude=np.ascontiguousarray(lat, np.float64), timestep=timestep, jul_start=jul_start)


# default routing1 parameters of mhm_parameter.nml (&routing1 'value' column)
ROUTING_PARAMS_DEFAULT = np.array([0.325, 0.075, 2.0, 0.1, 0.3])
ROUTING_PARAMS_BOUNDS = np.array([[0.31, 0.35], [0.07, 0.08], [1.95, 2.1], [0.09, 0.11], [0.01, 0.5]])


def make_eff_params(dom: Domain, seed: int = 3, lc_scale: float = 1.0) -> dict[str, np.ndarray]:
    """L1 effective parameters (the L1_* arrays mHM() reads) with realistic
    ranges: land-cover fractions from 5 synthetic classes mapped to mHM's
    forest / impervious / pervious codes, soil water capacities from per-horizon
    porosities, monthly interception capacity from 12 LAI classes."""
    rng = np.random.default_rng(seed)
    N, H = dom.n_cells, dom.n_horizons
    # 5 synthetic LC classes on 16 sub-cells per L1 cell -> {1 forest, 1, 3 pervious, 3, 2 impervious}
    cls = rng.integers(0, 5, (N, 16))
    f_forest = ((cls == 0) | (cls == 1)).mean(1)
    f_imp = (cls == 4).mean(1) * lc_scale
    f_sealed = 0.6 * f_imp                       # fracSealed_cityArea = 0.6
    f_perm = 1.0 - f_sealed - f_forest
    p: dict[str, np.ndarray] = {}
    p["fSealed"] = f_sealed
    p["tempThresh"] = np.full(N, 1.0) + rng.normal(0, 0.1, N)
    p["degDayNoPre"] = f_forest * 1.5 + f_sealed * 0.5 + f_perm * 0.5
    p["degDayMax"] = f_forest * 3.0 + f_sealed * 3.5 + f_perm * 4.0
    p["degDayInc"] = np.full(N, 0.5) * rng.uniform(0.8, 1.2, N)
    p["alpha"] = rng.uniform(0.10, 0.20, N)
    p["fAsp"] = rng.uniform(0.9, 1.1, N)
    p["HarSamCoeff"] = np.full(N, 0.0023)
    p["karstLoss"] = np.ones(N)
    p["kFastFlow"] = rng.uniform(1.5, 5.0, N)
    p["kSlowFlow"] = rng.uniform(5.0, 30.0, N)
    p["kPerco"] = rng.uniform(20.0, 80.0, N)
    k2 = rng.uniform(50.0, 300.0, N)
    p["kBaseFlow"] = np.maximum(k2, p["kSlowFlow"])  # mo_multi_param_reg.f90:618
    p["jarvis_thresh_c1"] = np.full(N, 0.5)
    p["unsatThresh"] = rng.uniform(20.0, 60.0, N)
    p["sealedThresh"] = np.full(N, 0.5)
    lai_class = rng.integers(0, 12, N)
    lai_tab = np.array([[0.5 + c * 0.4 + (2.0 + c * 0.3) * max(0.0, np.sin(np.pi * (m - 2) / 9.0))
                         for m in range(12)] for c in range(12)])
    lai = lai_tab[lai_class]                    # [N, 12]
    p["maxInter"] = np.ascontiguousarray((0.15 * lai).T.reshape(-1))  # (cell, month) column-major
    p["petLAIcorFactor"] = np.ascontiguousarray((0.3 + 0.8 * (1 - np.exp(-0.7 * lai))).T.reshape(-1))
    thick = np.diff(np.concatenate([[0.0], dom.horizon_depth]))
    por = rng.uniform(0.38, 0.50, (N, H))
    thfc = por * rng.uniform(0.55, 0.75, (N, H))
    thpw = thfc * rng.uniform(0.30, 0.55, (N, H))
    sms = por * thick[None, :]
    fc = thfc * thick[None, :]
    pw = thpw * thick[None, :]
    beta = rng.uniform(1.0, 4.0, (N, H))
    root = rng.uniform(0.90, 0.98, N)[:, None] ** (dom.horizon_depth[None, :] * 0.1)
    fr = np.diff(np.concatenate([np.ones((N, 1)), root], axis=1), axis=1) * -1.0
    fr = fr / fr.sum(1, keepdims=True)
    for name, arr in (("soilMoistSat", sms), ("soilMoistFC", fc), ("wiltingPoint", pw),
                      ("soilMoistExp", beta), ("fRoots", fr)):
        p[name] = np.ascontiguousarray(arr.T.reshape(-1))  # (cell, horizon) column-major
    for k in list(p):
        p[k] = np.ascontiguousarray(p[k], np.float64)
    return p


def _hargreaves_daily(tavg, tmax, tmin, lat_deg, doy):
    """Daily Hargreaves-Samani PET [mm d-1] for the forcing generator (the
    formula of pre-proc/hargreaves_samani_PET.py, with FAO-56 Ra)."""
    lat = np.deg2rad(lat_deg)
    dr = 1 + 0.033 * np.cos(2 * np.pi * doy / 365.0)
    dec = 0.409 * np.sin(2 * np.pi * doy / 365.0 - 1.39)
    ws = np.arccos(np.clip(-np.tan(lat) * np.tan(dec), -1, 1))
    ra = 24 * 60 / np.pi * 0.0820 * dr * (ws * np.sin(lat) * np.sin(dec) + np.cos(lat) * np.cos(dec) * np.sin(ws))
    return np.maximum(0.0, 0.0023 * ra * 0.408 * (tavg + 17.8) * np.sqrt(np.maximum(tmax - tmin, 0.0)))


def day_of_year(jul_start: int, day_index: np.ndarray) -> np.ndarray:
    """Day of year (1-based) of jul_start + day_index (Gregorian)."""
    J = jul_start + day_index
    f = J + 1401 + (((4 * J + 274277) // 146097) * 3) // 4 - 38
    e = 4 * f + 3
    g = (e % 1461) // 4
    h = 5 * g + 2
    m = ((h // 153 + 2) % 12) + 1
    y = e // 1461 - 4716 + (12 + 2 - m) // 12
    a = (14 - 1) // 12
    yy = y + 4800 - a
    mm = 1 + 12 * a - 3
    j0 = 1 + (153 * mm + 2) // 5 + 365 * yy + yy // 4 - yy // 100 + yy // 400 - 32045
    return J - j0 + 1


def make_forcing(dom: Domain, n_steps: int, seed: int = 2, t0: int = 1, dry_frac: float = 0.7,
                 gamma_k: float = 0.6, gamma_theta: float = 2.0) -> dict[str, np.ndarray]:
    """Hourly forcing rows t0..t0+n_steps-1, each [n_steps, N] float64:
    precipitation 70 % dry hours else Gamma(0.6, 2 mm/h), temperature
    8 + 10 sin(2 pi (doy - 81)/365) + N(0, 3) degC, PET Hargreaves-Samani from
    the day's temperature spread evenly over its hours."""
    rng = np.random.default_rng([seed, t0])
    N = dom.n_cells
    hours = np.arange(t0 - 1, t0 - 1 + n_steps) * dom.timestep
    day = hours // 24
    doy = day_of_year(dom.jul_start, day)
    wet = rng.random((n_steps, N)) >= dry_frac
    pre = np.where(wet, rng.gamma(gamma_k, gamma_theta, (n_steps, N)), 0.0)
    seas = 8.0 + 10.0 * np.sin(2 * np.pi * (doy - 81) / 365.0)
    temp = seas[:, None] + rng.normal(0.0, 3.0, (n_steps, N))
    # daily PET from the seasonal cycle +- 5 degC diurnal range, spread over 24 h
    pet_day = _hargreaves_daily(seas[:, None], seas[:, None] + 5.0, seas[:, None] - 5.0,
                                dom.latitude[None, :], doy[:, None])
    pet = pet_day / 24.0 * dom.timestep
    return {"pre": np.ascontiguousarray(pre), "temp": np.ascontiguousarray(temp),
            "pet": np.ascontiguousarray(pet)}


def make_forcing_grf(dom: Domain, n_steps: int, seed: int = 2, t0: int = 1, length_scale: float = 20.0,
                     dry_frac: float = 0.7, gamma_k: float = 0.6, gamma_theta: float = 2.0,
                     n_fields: int = 24, out: dict | None = None, threads: int = 0) -> dict[str, np.ndarray]:
    """Hourly forcing rows t0..t0+n_steps-1 with spatially correlated
    precipitation, each [n_steps, N] float64 (written into `out`'s arrays when
    given, e.g. pinned host buffers).

    Precipitation occurrence follows a Gaussian random field with a
    `length_scale`-cell correlation length (white noise filtered with a
    Gaussian kernel in Fourier space): a cell is wet where the field exceeds
    its 70 % quantile, and wet amounts are Gamma(0.6, 2 mm/h).  `n_fields`
    independent fields are generated per call and each step uses one of them
    shifted by a random offset on the periodic grid (a shifted stationary
    field has the same statistics), which keeps generation fast at 1e6
    cells.  Temperature 8 + 10 sin(2 pi (doy - 81)/365) + N(0, 3) degC; PET
    Hargreaves-Samani from the seasonal temperature with a 10 degC diurnal
    range, spread over the day's hours.  Every step draws from its own
    generator seeded with (seed, step), so the result is the same for any
    number of threads and on every machine (numpy's PCG64 and pocketfft)."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    nr, nc, N = dom.nrows, dom.ncols, dom.n_cells
    ky = np.fft.fftfreq(nr)[:, None]
    kx = np.fft.rfftfreq(nc)[None, :]
    filt = np.exp(-2.0 * (np.pi * length_scale) ** 2 * (kx * kx + ky * ky))
    nf = max(1, min(n_fields, n_steps))
    if out is None:
        out = {k: np.empty((n_steps, N)) for k in ("pre", "temp", "pet")}
    pre, temp, pet = out["pre"], out["temp"], out["pet"]
    hours = np.arange(t0 - 1, t0 - 1 + n_steps) * dom.timestep
    doy = day_of_year(dom.jul_start, hours // 24)
    seas = 8.0 + 10.0 * np.sin(2 * np.pi * (doy - 81) / 365.0)

    def field(i):
        w = np.random.default_rng([seed, t0, 17, i]).standard_normal((nr, nc))
        f = np.fft.irfft2(np.fft.rfft2(w) * filt, s=(nr, nc))
        return f, np.quantile(f, dry_frac)

    def step(t):
        rng = np.random.default_rng([seed, t0 + t, 18])
        f, thr = fields[t % nf]
        dy, dx = int(rng.integers(0, nr)), int(rng.integers(0, nc))
        wet = (np.roll(f, (dy, dx), axis=(0, 1)) > thr).T.reshape(-1)   # column-major pack
        row = pre[t]
        row[:] = 0.0
        row[wet] = rng.gamma(gamma_k, gamma_theta, int(wet.sum()))
        temp[t] = seas[t] + 3.0 * rng.standard_normal(N, dtype=np.float32)

    with ThreadPoolExecutor(max_workers=threads or min(32, os.cpu_count() or 1)) as ex:
        fields = list(ex.map(field, range(nf)))
        list(ex.map(step, range(n_steps)))
    days, first = np.unique(doy, return_index=True)
    for d, j in zip(days, first):
        pd = _hargreaves_daily(seas[j], seas[j] + 5.0, seas[j] - 5.0, dom.latitude, d) / 24.0 * dom.timestep
        pet[doy == d] = pd
    return out


def make_daily_forcing(dom: Domain, n_days: int, seed: int = 2, d0: int = 1) -> dict[str, np.ndarray]:
    """Daily forcing rows d0..d0+n_days-1 (for the day/night disaggregation and
    Hargreaves paths): pre [mm d-1], temp/tmin/tmax [degC], pet [mm d-1]."""
    rng = np.random.default_rng([seed, d0, 7])
    N = dom.n_cells
    day = np.arange(d0 - 1, d0 - 1 + n_days)
    doy = day_of_year(dom.jul_start, day)
    wet = rng.random((n_days, N)) >= 0.5
    pre = np.where(wet, rng.gamma(0.8, 6.0, (n_days, N)), 0.0)
    seas = 8.0 + 10.0 * np.sin(2 * np.pi * (doy - 81) / 365.0)
    temp = seas[:, None] + rng.normal(0.0, 3.0, (n_days, N))
    rngd = rng.uniform(3.0, 9.0, (n_days, N))
    tmin = temp - rngd / 2
    tmax = temp + rngd / 2
    pet = _hargreaves_daily(temp, tmax, tmin, dom.latitude[None, :], doy[:, None])
    return {k: np.ascontiguousarray(v, np.float64) for k, v in
            dict(pre=pre, temp=temp, tmin=tmin, tmax=tmax, pet=pet).items()}


@dataclass
class L0Maps:
    """Level-0 inputs of the parameter regionalisation (the fields of
    mhm_l0_desc), for an L1 grid subdivided `factor` x `factor`."""
    nrows0: int
    ncols0: int
    factor: int
    mask0: np.ndarray          # [ncols0 * nrows0] uint8, column-major
    l1_up: np.ndarray          # [N] int32 1-based L0 bounds of each L1 cell
    l1_down: np.ndarray
    l1_left: np.ndarray
    l1_right: np.ndarray
    l1_nsub: np.ndarray
    soil_id0: np.ndarray       # [N0] int32
    lcover0: np.ndarray        # [N0] int32 (1 forest, 2 sealed, 3 pervious)
    geo_unit0: np.ndarray      # [N0] int32
    slope0: np.ndarray         # [N0] degrees
    aspect0: np.ndarray        # [N0] degrees
    y0: np.ndarray             # [N0] latitude
    lai_class0: np.ndarray     # [N0] int32 1-based
    lai_lut: np.ndarray        # [n_lai, 12]
    soil_n_hor: np.ndarray     # [n_soil] int32
    soil_n_till: np.ndarray
    soil_ud: np.ndarray        # [n_soil, max_hor]
    soil_ld: np.ndarray
    soil_sand: np.ndarray
    soil_clay: np.ndarray
    soil_dbm: np.ndarray
    soil_rz_depth: np.ndarray  # [n_soil]
    geo_unit_list: np.ndarray  # [n_geo] int32
    geo_unit_kar: np.ndarray   # [n_geo] int32
    horizon_depth: np.ndarray  # [H]
    frac_sealed_city: float = 0.6
    lai_series: np.ndarray | None = None   # [n][N0] a gridded LAI series (replaces the table's 12 months)

    @property
    def n_cells0(self) -> int:
        return int(self.soil_id0.size)

    @property
    def n_soil(self) -> int:
        return int(self.soil_n_hor.size)

    @property
    def max_hor(self) -> int:
        return int(self.soil_ud.shape[1])

    @property
    def n_geo(self) -> int:
        return int(self.geo_unit_list.size)

    def lai0(self) -> np.ndarray:
        """Gridded LAI [entries][N0]: the series if set, else the look-up
        table expanded to [12][N0]."""
        if self.lai_series is not None:
            return np.ascontiguousarray(self.lai_series, np.float64)
        return np.ascontiguousarray(self.lai_lut[self.lai_class0 - 1].T)


LAI_LUT_12 = np.array([[0.5 + c * 0.4 + (2.0 + c * 0.3) * max(0.0, np.sin(np.pi * (m - 2) / 9.0))
                        for m in range(12)] for c in range(12)])


def make_l0(dom: Domain, factor: int = 4, seed: int = 4, n_soil: int = 10, holes: float = 0.0,
            lat_shift: float = 0.0, max_hor: int = 4) -> L0Maps:
    """L0 maps under the L1 grid of `dom`: 10 soil types with 2-4 layers
    (sand 5-90 %, clay 2-60 %, DbM 1.2-1.7, root-zone depth below the modelled
    horizons), 5 land-cover classes mapped to {1 forest, 1, 3 pervious, 3,
    2 sealed}, 12 LAI classes, 4 geological units (ids 1, 2, 4, 7; unit 4
    karstic; L0 cells may carry id 5, which maps to its nearest unit), slopes
    on a 0.1 degree grid (so ranks tie), aspect 0-360.  `holes` masks that
    fraction of L0 cells out (at least one stays in every L1 block)."""
    rng = np.random.default_rng(seed)
    nr, nc, f = dom.nrows, dom.ncols, factor
    nr0, nc0 = nr * f, nc * f
    H = dom.n_horizons
    # mask: full, minus random holes; keep each block's first cell
    mask2 = np.ones((nr0, nc0), bool)
    if holes > 0:
        mask2 &= rng.random((nr0, nc0)) >= holes
        mask2[::f, ::f] = True
    mask_cm = np.ascontiguousarray(mask2.T.reshape(-1)).astype(np.uint8)
    # L1 cell k (column-major over the full L1 grid): row k % nr, col k // nr
    k = np.arange(nr * nc)
    r1, c1 = k % nr, k // nr
    up = (r1 * f + 1).astype(np.int32)
    down = ((r1 + 1) * f).astype(np.int32)
    left = (c1 * f + 1).astype(np.int32)
    right = ((c1 + 1) * f).astype(np.int32)
    blocks = mask2.reshape(nr, f, nc, f).sum(axis=(1, 3))       # [nr, nc]
    nsub = np.ascontiguousarray(blocks.T.reshape(-1), np.int32)
    # packed L0 cells (column-major over the mask)
    rows0, cols0 = np.nonzero(mask2.T)                          # cols0 = row index, rows0 = col index
    ii, jj = cols0, rows0                                       # L0 row, col of each packed cell
    n0 = ii.size
    # soil types: coarse patches (3 L1 cells) with 20 % speckle
    pr, pc = max(1, nr0 // (3 * f)) + 1, max(1, nc0 // (3 * f)) + 1
    patch = rng.integers(1, n_soil + 1, (pr, pc))
    soil = patch[ii * pr // nr0, jj * pc // nc0]
    speck = rng.random(n0) < 0.2
    soil = np.where(speck, rng.integers(1, n_soil + 1, n0), soil).astype(np.int32)
    lc_map = np.array([1, 1, 3, 3, 2], np.int32)
    lcover = lc_map[rng.integers(0, 5, n0)]
    geo_list = np.array([1, 2, 4, 7], np.int32)
    geo = np.array([1, 2, 4, 5, 7], np.int32)[rng.integers(0, 5, n0)]
    slope = np.round(rng.uniform(0.0, 30.0, n0), 1)
    aspect = rng.uniform(0.0, 360.0, n0)
    lat = dom.latitude[(jj // f) * nr + (ii // f)] + lat_shift
    lai_class = rng.integers(1, 13, n0).astype(np.int32)
    # soil database
    hd = dom.horizon_depth.copy()
    top = hd[H - 2] if H >= 2 else 0.0
    nh = rng.integers(2, max_hor + 1, n_soil).astype(np.int32)
    ud = np.zeros((n_soil, max_hor))
    ld = np.zeros((n_soil, max_hor))
    rz = np.round(rng.uniform(top + 100.0, top + 1500.0, n_soil), -1)
    for s in range(n_soil):
        cuts = np.sort(rng.choice(np.arange(10.0, rz[s], 10.0), nh[s] - 1, replace=False))
        b = np.concatenate([[0.0], cuts, [rz[s]]])
        ud[s, :nh[s]] = b[:-1]
        ld[s, :nh[s]] = b[1:]
    ntill = np.minimum(nh, rng.integers(1, 3, n_soil)).astype(np.int32)
    sand = rng.uniform(5.0, 90.0, (n_soil, max_hor))
    clay = rng.uniform(2.0, 60.0, (n_soil, max_hor))
    clay = np.minimum(clay, np.maximum(2.0, 100.0 - sand))
    dbm = rng.uniform(1.2, 1.7, (n_soil, max_hor))
    c = np.ascontiguousarray
    return L0Maps(nrows0=nr0, ncols0=nc0, factor=f, mask0=mask_cm, l1_up=up, l1_down=down, l1_left=left,
                  l1_right=right, l1_nsub=nsub, soil_id0=c(soil), lcover0=c(lcover.astype(np.int32)),
                  geo_unit0=c(geo), slope0=c(slope), aspect0=c(aspect), y0=c(lat, np.float64),
                  lai_class0=c(lai_class), lai_lut=c(LAI_LUT_12), soil_n_hor=c(nh), soil_n_till=c(ntill),
                  soil_ud=c(ud), soil_ld=c(ld), soil_sand=c(sand), soil_clay=c(clay), soil_dbm=c(dbm),
                  soil_rz_depth=c(rz), geo_unit_list=geo_list, geo_unit_kar=np.array([0, 0, 1, 0], np.int32),
                  horizon_depth=c(hd))
