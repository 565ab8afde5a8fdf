"""ctypes binding of libmhm_gpu.so (the C ABI of include/mhm_gpu.h).

The library is built in-tree by mhm_gb300.build; loading fails loudly when it
is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import build as _build

MHM_OK = 0
MHM_ERR_INVALID = -1
MHM_ERR_CUDA = -2
MHM_ERR_OOM = -3
MHM_ERR_TIMEOUT = -4
MHM_ERR_NAN = -5
MHM_ERR_UNSUPPORTED = -6
MHM_ERR_BOUNDS = -7

FORC_PRE, FORC_TEMP, FORC_PET, FORC_TMIN, FORC_TMAX, FORC_NETRAD, FORC_EABS, FORC_WINDSPEED = range(8)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class DomainDesc(C.Structure):
    _fields_ = [
        ("n_cells", C.c_int32), ("n_horizons", C.c_int32), ("n_nodes", C.c_int32),
        ("n_outlets", C.c_int32), ("timestep", C.c_int32), ("proc_soilmoist", C.c_int32),
        ("proc_pet", C.c_int32), ("proc_routing", C.c_int32), ("n_tstep_forcing_day", C.c_int32),
        ("jul_start", C.c_int32), ("map_flag", C.c_int32), ("n_gauges", C.c_int32),
        ("n_members", C.c_int32), ("read_states", C.c_int32),
        ("evap_coeff", _dp), ("fday_prec", _dp), ("fnight_prec", _dp), ("fday_pet", _dp),
        ("fnight_pet", _dp), ("fday_temp", _dp), ("fnight_temp", _dp),
        ("l1_area_km2", _dp), ("l1_l11_id", _ip), ("l11_area_km2", _dp), ("l11_l1_id", _ip),
        ("net_perm", _ip), ("from_n", _ip), ("to_n", _ip),
        ("length", _dp), ("slope", _dp), ("ffp_imp", _dp), ("gauge_node", _ip), ("latitude", _dp),
    ]


EFF_PARAM_FIELDS = [
    "fSealed", "alpha", "degDayInc", "degDayMax", "degDayNoPre", "fAsp", "HarSamCoeff",
    "karstLoss", "kFastFlow", "kSlowFlow", "kBaseFlow", "kPerco",
    "jarvis_thresh_c1", "tempThresh", "unsatThresh", "sealedThresh",
    "maxInter", "petLAIcorFactor",
    "fRoots", "soilMoistSat", "soilMoistFC", "wiltingPoint", "soilMoistExp", "PrieTayAlpha",
    "aeroResist", "surfResist",
]


class EffParams(C.Structure):
    _fields_ = [(n, _dp) for n in EFF_PARAM_FIELDS]


RESTART_FIELDS = ["interc", "snowpack", "sealSTW", "unsatSTW", "satSTW", "soilMoist",
                  "qOUT", "Qmod", "qTIN", "qTR", "C1", "C2"]


class Restart(C.Structure):
    _fields_ = [(n, _dp) for n in RESTART_FIELDS]


class L0Desc(C.Structure):
    """mhm_l0_desc: level-0 inputs of the parameter regionalisation."""
    _fields_ = [
        ("n_cells0", C.c_int32), ("nrows0", C.c_int32), ("ncols0", C.c_int32), ("n_soil_types", C.c_int32),
        ("max_soil_hor", C.c_int32), ("n_geo_units", C.c_int32), ("n_lai_classes", C.c_int32), ("n_lai_steps", C.c_int32),
        ("frac_sealed_city", C.c_double), ("horizon_depth", _dp), ("mask0", C.POINTER(C.c_uint8)),
        ("l1_up", _ip), ("l1_down", _ip), ("l1_left", _ip), ("l1_right", _ip), ("l1_nsub", _ip),
        ("soil_id0", _ip), ("lcover0", _ip), ("geo_unit0", _ip), ("slope0", _dp), ("aspect0", _dp), ("y0", _dp),
        ("lai_class0", _ip), ("lai_lut", _dp), ("lai0", _dp), ("soil_n_hor", _ip), ("soil_n_till", _ip),
        ("soil_ud", _dp), ("soil_ld", _dp), ("soil_sand", _dp), ("soil_clay", _dp), ("soil_dbm", _dp),
        ("soil_rz_depth", _dp), ("geo_unit_list", _ip), ("geo_unit_kar", _ip),
    ]


class LaunchConfig(C.Structure):
    """mhm_launch_config."""
    _fields_ = [("cell_blocks_per_sm", C.c_int32), ("route_sub_steps", C.c_int32), ("chunk_steps", C.c_int32),
                ("route_cluster", C.c_int32)]


class L0Flow(C.Structure):
    """mhm_l0_flow: level-0 flow data of a basin."""
    _fields_ = [("nrows0", C.c_int32), ("ncols0", C.c_int32), ("factor", C.c_int32), ("n_cells0", C.c_int32),
                ("mask0", C.POINTER(C.c_uint8)), ("fdir0", _ip), ("facc0", _ip), ("elev0", _dp),
                ("cellsize0", C.c_double), ("n_lc_scenes", C.c_int32), ("lc_class_imp", C.c_int32),
                ("lcover0", _ip)]


class L11Network(C.Structure):
    """mhm_l11_network: the network mRM's start-up derives."""
    _fields_ = [("n_nodes", C.c_int32), ("n_outlets", C.c_int32), ("n_links", C.c_int32), ("nrows11", C.c_int32),
                ("ncols11", C.c_int32), ("n_l0_outlets", C.c_int32)] + \
               [(n, _ip) for n in ("fdir11", "cell_row11", "cell_col11", "from_n", "to_n", "net_perm", "r_order",
                                   "row_out", "col_out")] + \
               [(n, _dp) for n in ("length", "slope", "a_floodplain", "frac_fp_imp")]


class OutputConfig(C.Structure):
    """mhm_output_config: aggregated flux/state (or Qrouted) outputs."""
    _fields_ = [
        ("timestep_model_outputs", C.c_int32), ("max_slots", C.c_int32), ("warming_steps", C.c_int64),
        ("n_time_steps", C.c_int64), ("flags", C.c_int32 * 21), ("pad_", C.c_int32),
    ]


EXPORTS = [
    "mhm_ctx_create", "mhm_ctx_destroy", "mhm_last_error", "mhm_ctx_stream", "mhm_set_eff_params",
    "mhm_set_routing_params", "mhm_init_states", "mhm_set_forcing", "mhm_run", "mhm_enable_outputs",
    "mhm_get_outputs", "mhm_get_state", "mhm_set_state", "mhm_get_var", "mhm_set_timing",
    "mhm_get_timing", "mhm_host_alloc", "mhm_host_free", "mhm_version", "mhm_kernel_launch_count",
    "mhm_hmath_eval", "mhm_probe_fp64", "mhm_routing_order", "mhm_step_calendar", "mhm_run_async", "mhm_sync",
    "mhm_mpr_setup", "mhm_gamma_layout", "mhm_mpr", "mhm_mpr_get_aux", "mhm_get_eff_params",
    "mhm_soil_weights", "mhm_slope_emp", "mhm_mpr_noalloc",
    "mhm_run_members_async", "mhm_snapshot_alloc", "mhm_snapshot_save", "mhm_snapshot_load", "mhm_autotune",
    "mhm_enable_fluxes", "mhm_get_fluxes", "mhm_set_link_fpimp",
    "mhm_enable_flux_state_outputs", "mhm_read_flux_state_outputs", "mhm_enable_routed_outputs",
    "mhm_read_routed_outputs", "mhm_set_output_weights", "mhm_set_link_celerity", "mhm_network_topology",
    "mhm_poll", "mhm_set_meteo_weights", "mhm_set_inflow_gauges", "mhm_set_inflow_discharge",
    "mhm_member_status", "mhm_set_launch_config", "mhm_get_launch_config", "mhm_autotune_ex",
    "mhm_batch_create", "mhm_batch_destroy", "mhm_batch_last_error", "mhm_batch_run_members",
    "mhm_l11_network_size", "mhm_l11_network", "mhm_l1_l11_mapping", "mhm_autotune_route",
    "mhm_bounds_checked", "mhm_device_status", "mhm_bounds_selftest", "mhm_set_lai_series", "mhm_set_lai_params",
    "mhm_step_lai", "mhm_get_lai_params",
]

_LIB = None


def bounds_checked_requested() -> bool:
    """MHM_BOUNDS_CHECK=1 selects the bounds-checked build (libmhm_gpu_bc.so)."""
    return os.environ.get("MHM_BOUNDS_CHECK", "0") not in ("", "0")


def lib_path() -> Path:
    return _build.LIB_BC if bounds_checked_requested() else _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libmhm_gpu.so (building it first if needed); raises if unavailable."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if build_if_missing and (not path.exists() or _build._stale(path)):
        _build.build(bounds_check=bounds_checked_requested())
    if not path.exists():
        raise RuntimeError(f"libmhm_gpu.so not found at {path}: run mhm_gb300.build.build()")
    L = C.CDLL(str(path), mode=os.RTLD_NOW | getattr(os, "RTLD_GLOBAL", 0))
    vp = C.c_void_p
    L.mhm_ctx_create.argtypes = [C.POINTER(DomainDesc), C.c_int32, C.POINTER(vp)]
    L.mhm_ctx_destroy.argtypes = [vp]
    L.mhm_last_error.argtypes = [vp]
    L.mhm_last_error.restype = C.c_char_p
    L.mhm_ctx_stream.argtypes = [vp]
    L.mhm_ctx_stream.restype = vp
    L.mhm_set_eff_params.argtypes = [vp, C.c_int32, C.POINTER(EffParams)]
    L.mhm_get_eff_params.argtypes = [vp, C.c_int32, C.POINTER(EffParams)]
    L.mhm_set_routing_params.argtypes = [vp, C.c_int32, _dp]
    L.mhm_init_states.argtypes = [vp, C.c_int32, _dp]
    L.mhm_set_forcing.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, vp, C.c_int32]
    L.mhm_run.argtypes = [vp, C.c_int32, C.c_int32, _dp]
    L.mhm_run_async.argtypes = [vp, C.c_int32, C.c_int32, _dp]
    L.mhm_sync.argtypes = [vp]
    L.mhm_enable_outputs.argtypes = [vp, C.c_int32, C.c_int32]
    L.mhm_get_outputs.argtypes = [vp, _dp, _dp]
    L.mhm_get_state.argtypes = [vp, C.c_int32, C.POINTER(Restart)]
    L.mhm_set_state.argtypes = [vp, C.c_int32, C.POINTER(Restart)]
    L.mhm_get_var.argtypes = [vp, C.c_int32, C.c_char_p, _dp]
    L.mhm_set_timing.argtypes = [vp, C.c_int32]
    L.mhm_get_timing.argtypes = [vp, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
    L.mhm_host_alloc.argtypes = [C.c_size_t, C.POINTER(vp)]
    L.mhm_host_free.argtypes = [vp]
    L.mhm_version.argtypes = [_ip, _ip]
    L.mhm_kernel_launch_count.argtypes = []
    L.mhm_kernel_launch_count.restype = C.c_int64
    L.mhm_hmath_eval.argtypes = [C.c_int32, C.c_int32, C.c_int64, _dp, _dp, _dp]
    L.mhm_probe_fp64.argtypes = [C.c_int64, C.POINTER(C.c_double)]
    L.mhm_routing_order.argtypes = [C.c_int32, C.c_int32, _ip, _ip, _ip, _ip]
    L.mhm_step_calendar.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, _ip, _ip, _ip]
    L.mhm_mpr_setup.argtypes = [vp, C.POINTER(L0Desc)]
    L.mhm_gamma_layout.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, _ip]
    L.mhm_mpr.argtypes = [vp, C.c_int32, C.c_int32, _dp, C.c_int32]
    L.mhm_mpr_get_aux.argtypes = [vp, C.c_char_p, _dp]
    L.mhm_soil_weights.argtypes = [C.c_int32, C.c_int32, _ip, _dp, _dp, _dp, C.c_int32, _dp, _dp]
    L.mhm_slope_emp.argtypes = [C.c_int32, _dp, _dp]
    L.mhm_mpr_noalloc.argtypes = [vp, C.c_int32, _dp, C.c_int32]
    L.mhm_run_members_async.argtypes = [vp, _ip, C.c_int32, _dp]
    L.mhm_snapshot_alloc.argtypes = [vp, C.c_int32]
    L.mhm_autotune.argtypes = [vp, C.c_int32, C.c_int32, _ip, _ip, _dp]
    L.mhm_enable_fluxes.argtypes = [vp, C.c_int32]
    L.mhm_set_link_fpimp.argtypes = [vp, _dp]
    L.mhm_set_meteo_weights.argtypes = [vp, _dp, _dp, _dp]
    L.mhm_get_fluxes.argtypes = [vp, _dp, _dp]
    L.mhm_snapshot_save.argtypes = [vp, C.c_int32, C.c_int32]
    i64p = C.POINTER(C.c_int64)
    L.mhm_enable_flux_state_outputs.argtypes = [vp, C.POINTER(OutputConfig)]
    L.mhm_enable_routed_outputs.argtypes = [vp, C.POINTER(OutputConfig)]
    L.mhm_read_flux_state_outputs.argtypes = [vp, _dp, i64p, C.c_int32, _ip, _ip]
    L.mhm_read_routed_outputs.argtypes = [vp, _dp, i64p, C.c_int32, _ip]
    L.mhm_set_output_weights.argtypes = [vp, C.c_int32, C.c_int64, _dp, _dp]
    L.mhm_set_link_celerity.argtypes = [vp, C.c_int32, _dp]
    L.mhm_poll.argtypes = [vp, _ip]
    L.mhm_network_topology.argtypes = [C.c_int32, C.c_int32, _ip, C.c_int32, _ip, _ip, _ip, _ip, _ip, _ip]
    L.mhm_snapshot_load.argtypes = [vp, C.c_int32, C.c_int32]
    L.mhm_set_inflow_gauges.argtypes = [vp, C.c_int32, _ip, _ip]
    L.mhm_set_inflow_discharge.argtypes = [vp, C.c_int32, C.c_int32, _dp]
    L.mhm_member_status.argtypes = [vp, _ip]
    L.mhm_set_launch_config.argtypes = [vp, C.POINTER(LaunchConfig)]
    L.mhm_get_launch_config.argtypes = [vp, C.POINTER(LaunchConfig)]
    L.mhm_autotune_ex.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, _ip, C.POINTER(LaunchConfig), _dp]
    L.mhm_autotune_route.argtypes = [vp, C.c_int32, C.c_int32, _ip, _dp]
    L.mhm_bounds_checked.argtypes = []
    L.mhm_device_status.argtypes = [vp, _ip, C.POINTER(C.c_int64)]
    L.mhm_bounds_selftest.argtypes = [vp]
    L.mhm_set_lai_series.argtypes = [vp, C.c_int32, C.c_int32]
    L.mhm_set_lai_params.argtypes = [vp, C.c_int32, _dp, _dp, _dp]
    L.mhm_step_lai.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _ip]
    L.mhm_get_lai_params.argtypes = [vp, C.c_int32, _dp, _dp, _dp]
    L.mhm_batch_create.argtypes = [C.c_int32, C.POINTER(vp)]
    L.mhm_batch_destroy.argtypes = [vp]
    L.mhm_batch_last_error.argtypes = [vp]
    L.mhm_batch_last_error.restype = C.c_char_p
    L.mhm_batch_run_members.argtypes = [vp, C.c_int32, C.POINTER(vp), C.POINTER(_ip), C.c_int32, C.POINTER(_dp)]
    L.mhm_l11_network_size.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_uint8), C.c_int32, _ip]
    L.mhm_l11_network.argtypes = [C.POINTER(L0Flow), C.POINTER(L11Network)]
    L.mhm_l1_l11_mapping.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_uint8), C.c_int32, C.c_int32, _ip, _ip]
    _LIB = L
    return L
