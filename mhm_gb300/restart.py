"""Restart files in the reference's layout.

mHM writes one restart file per domain with the L1 states, the fluxes of the
last step and the effective parameters of every land-cover scene
(write_restart_files, src/mHM/mo_restart.f90:53-258, write_eff_params,
src/MPR/mo_mpr_restart.f90:159-300); mRM writes the L11 network, routing
states and Muskingum coefficients (mrm_write_restart,
src/mRM/mo_mrm_restart.f90:56-418).  A run started from them reads the
states and parameters instead of running MPR and initialising the soil
moisture (read_restart_states, src/mHM/mo_restart.f90:292-821;
mhm_interface_run_prepare, src/mHM/mo_mhm_interface_run.f90:221-236).

Grids are stored with netCDF dimensions (..., ncols, nrows) -- Fortran's
(nrows, ncols, ...) reversed -- and cell vectors are packed over the mask
in that row-major order, which is Fortran's column-major pack.  Reading
takes the reference's netCDF-4 files (through h5read) and classic /
64-bit-offset netCDF files; writing produces 64-bit-offset netCDF, which
the reference's netCDF library reads as well.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

NODATA = -9999.0   # nodata_dp, src/common/mo_common_constants.f90

# mHM restart variable -> (mhm_eff_params name, leading dimensions before the grid)
EFF_PARAMS = {
    "L1_fSealed": ("fSealed", ("scene",)),
    "L1_alpha": ("alpha", ("scene",)),
    "L1_degDayInc": ("degDayInc", ("scene",)),
    "L1_degDayMax": ("degDayMax", ("scene",)),
    "L1_degDayNoPre": ("degDayNoPre", ("scene",)),
    "L1_karstLoss": ("karstLoss", ()),
    "L1_fRoots": ("fRoots", ("scene", "horizon")),
    "L1_maxInter": ("maxInter", ("lai",)),
    "L1_kfastFlow": ("kFastFlow", ("scene",)),
    "L1_kSlowFlow": ("kSlowFlow", ("scene",)),
    "L1_kBaseFlow": ("kBaseFlow", ("scene",)),
    "L1_kPerco": ("kPerco", ("scene",)),
    "L1_soilMoistFC": ("soilMoistFC", ("scene", "horizon")),
    "L1_soilMoistSat": ("soilMoistSat", ("scene", "horizon")),
    "L1_soilMoistExp": ("soilMoistExp", ("scene", "horizon")),
    "L1_jarvis_thresh_c1": ("jarvis_thresh_c1", ()),
    "L1_petLAIcorFactor": ("petLAIcorFactor", ("scene", "lai")),
    "L1_tempThresh": ("tempThresh", ("scene",)),
    "L1_unsatThresh": ("unsatThresh", ()),
    "L1_sealedThresh": ("sealedThresh", ()),
    "L1_wiltingPoint": ("wiltingPoint", ("scene", "horizon")),
    "L1_fAsp": ("fAsp", ()),
    "L1_HarSamCoeff": ("HarSamCoeff", ()),
    "L1_PrieTayAlpha": ("PrieTayAlpha", ("lai",)),
    "L1_aeroResist": ("aeroResist", ("scene", "lai")),
    "L1_surfResist": ("surfResist", ("lai",)),
}
# mHM restart variable -> state name of mhm_restart (the L1 storages)
STATES = {"L1_Inter": "interc", "L1_snowPack": "snowpack", "L1_sealSTW": "sealSTW", "L1_soilMoist": "soilMoist",
          "L1_unsatSTW": "unsatSTW", "L1_satSTW": "satSTW"}
LONG_NAMES = {
    "L1_Inter": "Interception storage at level 1", "L1_snowPack": "Snowpack at level 1",
    "L1_sealSTW": "Retention storage of impervious areas at level 1", "L1_soilMoist": "soil moisture at level 1",
    "L1_unsatSTW": "upper soil storage at level 1", "L1_satSTW": "groundwater storage at level 1",
}
# mRM restart: routing states / coefficients over the L11 cells, and the network per link
MRM_STATES = {"L11_qOUT": "qOUT", "L11_Qmod": "Qmod", "L11_qTIN": "qTIN", "L11_qTR": "qTR", "L11_C1": "C1",
              "L11_C2": "C2"}
MRM_LINK_INT = ("L11_fromN", "L11_toN", "L11_rOrder", "L11_netPerm")
MRM_LINK_DP = ("L11_length", "L11_slope")


def read_dataset(path) -> dict[str, np.ndarray]:
    """Every readable variable of a netCDF file (netCDF-4 / HDF5 or classic)."""
    with open(path, "rb") as f:
        magic = f.read(4)
    if magic == b"\x89HDF":
        from . import h5read
        h = h5read.H5File(str(path))
        out = {}
        for name in h.group():
            try:
                out[name] = h.read(name)
            except (NotImplementedError, ValueError):
                pass   # netCDF dimension scales without values
        return out
    if magic[:3] == b"CDF":
        from scipy.io import netcdf_file
        with netcdf_file(str(path), "r", mmap=False) as f:
            return {k: np.array(v.data) for k, v in f.variables.items()}
    raise ValueError(f"{path}: not a netCDF file")


def _pack(grid: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """[..., ncols, nrows] -> [..., n_cells] over the mask."""
    return np.ascontiguousarray(grid[..., mask])


def _unpack(cells: np.ndarray, mask: np.ndarray) -> np.ndarray:
    cells = np.asarray(cells, np.float64)
    out = np.full(cells.shape[:-1] + mask.shape, NODATA)
    out[..., mask] = cells
    return out


@dataclass
class MhmRestart:
    """An mHM restart: the L1 mask, states packed over it and the effective
    parameters of every land-cover scene."""
    mask: np.ndarray                                  # [ncols1][nrows1] bool
    states: dict[str, np.ndarray]                     # mhm_restart names, [n_cells] / [H][n_cells]
    params: dict[str, np.ndarray]                     # mhm_eff_params names, [scene?][horizon|lai?][n_cells]
    horizon_depth: np.ndarray                         # lower bound of each soil horizon [mm]
    n_scenes: int = 1
    extra: dict[str, np.ndarray] = field(default_factory=dict)

    @property
    def n_lai(self) -> int:
        """LAI entries of the LAI-indexed parameters (L1_LAITimesteps): 12
        monthly slots, or the length of a gridded LAI series."""
        a = self.params.get("maxInter")
        return int(a.shape[0]) if a is not None and a.ndim == 2 else 12

    def lai_params(self, scene: int = 0) -> dict[str, np.ndarray]:
        """The scene's LAI-indexed parameters, each [n_lai][n_cells]."""
        out = {}
        for var, (name, dims) in EFF_PARAMS.items():
            if "lai" not in dims or name not in self.params:
                continue
            a = self.params[name]
            if dims[0] == "scene":
                a = a[min(scene, a.shape[0] - 1)]
            out[name] = np.ascontiguousarray(a, np.float64)
        return out

    def eff_params(self, scene: int = 0) -> dict[str, np.ndarray]:
        """The scene's parameters as mhm_set_eff_params takes them (flattened)."""
        out = {}
        for var, (name, dims) in EFF_PARAMS.items():
            if name not in self.params:
                continue
            a = self.params[name]
            if dims and dims[0] == "scene":
                a = a[min(scene, a.shape[0] - 1)]
            out[name] = np.ascontiguousarray(a, np.float64).reshape(-1)
        return out


def read_mhm_restart(path) -> MhmRestart:
    ds = read_dataset(path)
    mask = ds["L1_domain_mask"].astype(bool)
    states = {STATES[k]: _pack(ds[k], mask) for k in STATES}
    states["soilMoist"] = states["soilMoist"].reshape(-1)
    params = {name: _pack(ds[var], mask) for var, (name, _) in EFF_PARAMS.items() if var in ds}
    bnds = ds.get("L1_SoilHorizons_bnds")
    hd = np.asarray(bnds[:, 1], np.float64) if bnds is not None else np.zeros(0)
    n_scenes = int(ds["L1_fSealed"].shape[0]) if ds.get("L1_fSealed") is not None and ds["L1_fSealed"].ndim == 3 \
        else 1
    extra = {k: v for k, v in ds.items() if k.startswith("L1_") and k not in STATES and k not in EFF_PARAMS}
    return MhmRestart(mask, states, params, hd, n_scenes, extra)


@dataclass
class MrmRestart:
    """An mRM restart: the L11 mask, routing states (by L11 node, links first)
    and the network of links."""
    mask: np.ndarray                                  # [ncols11][nrows11] bool
    states: dict[str, np.ndarray]                     # qOUT, Qmod [L]; qTIN, qTR [2 * L]; C1, C2 [L]
    network: dict[str, np.ndarray]
    ts_rout: float | None = None


def read_mrm_restart(path) -> MrmRestart:
    ds = read_dataset(path)
    mask = ds["L11_domain_mask"].astype(bool)
    states = {name: _pack(ds[var], mask).reshape(-1) for var, name in MRM_STATES.items() if var in ds}
    net = {}
    for k in MRM_LINK_INT:
        if k in ds:
            net[k[4:]] = np.asarray(ds[k], np.int32)
    n_links = int((net["fromN"] > 0).sum()) if "fromN" in net else 0   # outlets carry nodata
    for k in MRM_LINK_DP:
        if k in ds:
            net[k[4:]] = np.asarray(ds[k][:n_links], np.float64)
    if "L11_nLinkFracFPimp" in ds:
        ffp = ds["L11_nLinkFracFPimp"]
        net["fFPimp"] = np.stack([_pack(ffp[s], mask)[:n_links] for s in range(ffp.shape[0])])
    for k in ("L1_L11_Id", "L11_L1_Id"):
        if k in ds:
            src_mask = ds["L1_domain_mask"].astype(bool) if k.startswith("L1_") else mask
            net[k] = _pack(ds[k], src_mask).astype(np.int32)
    if "gaugeNodeList" in ds:
        net["gaugeNodeList"] = np.asarray(ds["gaugeNodeList"], np.int32).reshape(-1)
    ts = float(np.asarray(ds["L11_TSrout"]).reshape(-1)[0]) if "L11_TSrout" in ds else None
    return MrmRestart(mask, states, net, ts)


def process_params(proc_sm: int, proc_pet: int) -> set[str]:
    """The process-dependent restart variables the reference writes for
    processCase(3) = proc_sm and processCase(5) = proc_pet
    (src/MPR/mo_mpr_restart.f90:257-312): the Jarvis threshold for soil
    moisture cases 2 and 3; per PET case the LAI correction factor (-1),
    the aspect factor (-1, 0, 1), the Hargreaves-Samani coefficient (1),
    the Priestley-Taylor alpha (2) or the aerodynamic and bulk surface
    resistances (3)."""
    out = set()
    if proc_sm in (2, 3):
        out.add("L1_jarvis_thresh_c1")
    if proc_pet == -1:
        out.add("L1_petLAIcorFactor")
    if proc_pet in (-1, 0, 1):
        out.add("L1_fAsp")
    if proc_pet == 1:
        out.add("L1_HarSamCoeff")
    if proc_pet == 2:
        out.add("L1_PrieTayAlpha")
    if proc_pet == 3:
        out |= {"L1_aeroResist", "L1_surfResist"}
    return out


PROCESS_DEPENDENT = {"L1_jarvis_thresh_c1", "L1_petLAIcorFactor", "L1_fAsp", "L1_HarSamCoeff", "L1_PrieTayAlpha",
                     "L1_aeroResist", "L1_surfResist"}


def write_mhm_restart(path, mask: np.ndarray, states: dict[str, np.ndarray], params_by_scene: list[dict],
                      horizon_depth, lai_bounds=None, proc_sm: int | None = None,
                      proc_pet: int | None = None) -> None:
    """The states and the effective parameters of every scene in the layout
    of write_restart_files / write_eff_params (64-bit-offset netCDF).
    `states` as mhm_get_state returns them, `params_by_scene` one
    mhm_eff_params dict per land-cover scene (flattened arrays).  With the
    process cases given, the process-dependent parameters are the ones the
    reference writes for them (process_params); otherwise every parameter
    present in all scenes is written."""
    keep = None if proc_sm is None or proc_pet is None else process_params(proc_sm, proc_pet)
    from scipy.io import netcdf_file
    mask = np.asarray(mask, bool)
    n = int(mask.sum())
    hd = np.asarray(horizon_depth, np.float64)
    H = hd.size
    S = len(params_by_scene)
    # LAI entries: 12 monthly slots, or the length of a gridded LAI series
    mi = params_by_scene[-1].get("maxInter")
    n_lai = int(np.asarray(mi).size // n) if mi is not None else 12
    with netcdf_file(str(path), "w", version=2) as f:
        f.createDimension("ncols1", mask.shape[0])
        f.createDimension("nrows1", mask.shape[1])
        f.createDimension("L1_SoilHorizons", H)
        f.createDimension("L1_LandCoverPeriods", S)
        f.createDimension("L1_LAITimesteps", n_lai)
        f.createDimension("bnds", 2)
        v = f.createVariable("L1_domain_mask", "i4", ("ncols1", "nrows1"))
        v[:] = mask.astype(np.int32)
        v = f.createVariable("L1_SoilHorizons_bnds", "f8", ("L1_SoilHorizons", "bnds"))
        v[:] = np.stack([np.concatenate([[0.0], hd[:-1]]), hd], axis=1)
        if lai_bounds is not None:
            v = f.createVariable("L1_LAITimesteps_bnds", "f8", ("L1_LAITimesteps", "bnds"))
            v[:] = np.asarray(lai_bounds, np.float64)

        def put(name, cells, dims, long_name=None):
            var = f.createVariable(name, "f8", dims + ("ncols1", "nrows1"))
            var._FillValue = NODATA
            var[:] = _unpack(np.asarray(cells, np.float64).reshape(*[f.dimensions[d] for d in dims], n), mask)
            if long_name:
                var.long_name = long_name
        for var, name in STATES.items():
            put(var, states[name], ("L1_SoilHorizons",) if name == "soilMoist" else (), LONG_NAMES[var])
        dim_of = {"scene": "L1_LandCoverPeriods", "horizon": "L1_SoilHorizons", "lai": "L1_LAITimesteps"}
        for var, (name, dims) in EFF_PARAMS.items():
            if any(name not in p or p[name] is None for p in params_by_scene):
                continue
            if keep is not None and var in PROCESS_DEPENDENT and var not in keep:
                continue
            if dims and dims[0] == "scene":
                cells = np.stack([np.asarray(p[name], np.float64) for p in params_by_scene])
            else:
                cells = np.asarray(params_by_scene[-1][name], np.float64)
            put(var, cells, tuple(dim_of[d] for d in dims))


def write_mrm_restart(path, mask: np.ndarray, states: dict[str, np.ndarray], network: dict[str, np.ndarray],
                      ts_rout: float | None = None, mask1: np.ndarray | None = None) -> None:
    """Routing states, Muskingum coefficients and the link network in the
    layout of mrm_write_restart (64-bit-offset netCDF); `states` as
    mhm_get_state returns them (by L11 node), `network` with the keys
    read_mrm_restart gives (fromN, toN, rOrder, netPerm, length, slope,
    fFPimp [scene][link], L11_L1_Id, gaugeNodeList; L1_L11_Id with the L1
    mask `mask1`)."""
    from scipy.io import netcdf_file
    mask = np.asarray(mask, bool)
    n = int(mask.sum())
    with netcdf_file(str(path), "w", version=2) as f:
        f.createDimension("ncols11", mask.shape[0])
        f.createDimension("nrows11", mask.shape[1])
        f.createDimension("nIT", 2)
        f.createDimension("nLinks", n)
        v = f.createVariable("L11_domain_mask", "i4", ("ncols11", "nrows11"))
        v[:] = mask.astype(np.int32)
        for var, name in MRM_STATES.items():
            if name not in states:
                continue
            a = np.asarray(states[name], np.float64)
            dims = ("nIT",) if name in ("qTIN", "qTR") else ()
            x = f.createVariable(var, "f8", dims + ("ncols11", "nrows11"))
            x._FillValue = NODATA
            x[:] = _unpack(a.reshape(*([2] if dims else []), n), mask)
        for k in MRM_LINK_INT:
            if k[4:] in network:
                x = f.createVariable(k, "i4", ("nLinks",))
                a = np.full(n, -9999, np.int32)
                src = np.asarray(network[k[4:]], np.int32)
                a[: src.size] = src
                x[:] = a
        for k in MRM_LINK_DP:
            if k[4:] in network:
                x = f.createVariable(k, "f8", ("nLinks",))
                a = np.full(n, NODATA)
                src = np.asarray(network[k[4:]], np.float64)
                a[: src.size] = src
                x[:] = a
        if "fFPimp" in network:
            ffp = np.atleast_2d(np.asarray(network["fFPimp"], np.float64))
            f.createDimension("L1_LandCoverPeriods", ffp.shape[0])
            x = f.createVariable("L11_nLinkFracFPimp", "f8", ("L1_LandCoverPeriods", "ncols11", "nrows11"))
            x._FillValue = NODATA
            full = np.zeros((ffp.shape[0], n))
            full[:, : ffp.shape[1]] = ffp
            x[:] = _unpack(full, mask)
        if "L11_L1_Id" in network:
            x = f.createVariable("L11_L1_Id", "i4", ("ncols11", "nrows11"))
            g = np.full(mask.shape, -9999, np.int32)
            g[mask] = np.asarray(network["L11_L1_Id"], np.int32)
            x[:] = g
        if "L1_L11_Id" in network and mask1 is not None:
            m1 = np.asarray(mask1, bool)
            f.createDimension("ncols1", m1.shape[0])
            f.createDimension("nrows1", m1.shape[1])
            x = f.createVariable("L1_domain_mask", "i4", ("ncols1", "nrows1"))
            x[:] = m1.astype(np.int32)
            x = f.createVariable("L1_L11_Id", "i4", ("ncols1", "nrows1"))
            g = np.full(m1.shape, -9999, np.int32)
            g[m1] = np.asarray(network["L1_L11_Id"], np.int32)
            x[:] = g
        if "gaugeNodeList" in network:
            gn = np.asarray(network["gaugeNodeList"], np.int32).reshape(-1)
            f.createDimension("Ngauges", gn.size)
            x = f.createVariable("gaugeNodeList", "i4", ("Ngauges",))
            x[:] = gn
        if ts_rout is not None:
            f.createDimension("TS", 1)
            x = f.createVariable("L11_TSrout", "i4", ("TS",))
            x[:] = np.array([int(ts_rout)], np.int32)
