"""Host-side interface over the C ABI, shaped like the reference's run API.

The reference drives one basin with mhm_interface_run_prepare /
prepare_domain / do_time_step (src/mHM/mo_mhm_interface_run.f90:160-638) and
exposes them to Python as ``mhm.run.*`` (pybind/src/wrapper.f90:176-233).
``MhmGpu`` keeps that vocabulary: ``prepare`` loads effective parameters and
default states (the restart path of mhm_interface_run_prepare), ``set_meteo``
hands over forcing, ``run`` advances time steps (do_time_step x n) and
``get_variable`` / ``get_runoff`` read results back.  Everything executes in
libmhm_gpu.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib, outputs
from .synth import Domain

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def _d(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _i(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


class MhmError(RuntimeError):
    pass


class MhmGpu:
    """One basin (optionally with n_members parameter sets) on one GPU."""

    def __init__(self, dom: Domain, proc_soilmoist: int = 1, proc_pet: int = 0, proc_routing: int = 1,
                 hourly: bool = True, n_members: int = 1, read_states: bool = False, device: int = -1):
        self.L = _lib.load()
        self.dom = dom
        self.n_members = n_members
        self._lai = (0, 12)      # (timeStep_LAI_input, LAI entries) of the context
        self._keep: list = []

        def keep(a, dt=np.float64):
            a = np.ascontiguousarray(a, dt)
            self._keep.append(a)
            return a

        d = _lib.DomainDesc()
        d.n_cells = dom.n_cells
        d.n_horizons = dom.n_horizons
        d.n_nodes = dom.n_nodes
        d.n_outlets = dom.n_outlets
        d.timestep = dom.timestep
        d.proc_soilmoist = proc_soilmoist
        d.proc_pet = proc_pet
        d.proc_routing = proc_routing
        self.proc_soilmoist, self.proc_pet = proc_soilmoist, proc_pet
        d.n_tstep_forcing_day = 24 if hourly else 1
        d.jul_start = dom.jul_start
        d.map_flag = 1
        d.n_gauges = len(dom.gauge_node)
        d.n_members = n_members
        d.read_states = 1 if read_states else 0
        d.evap_coeff = _d(keep(dom.evap_coeff))
        d.fday_prec = _d(keep(dom.fday_prec))
        d.fnight_prec = _d(keep(dom.fnight_prec))
        d.fday_pet = _d(keep(dom.fday_pet))
        d.fnight_pet = _d(keep(dom.fnight_pet))
        d.fday_temp = _d(keep(dom.fday_temp))
        d.fnight_temp = _d(keep(dom.fnight_temp))
        d.l1_area_km2 = _d(keep(dom.l1_area_km2))
        d.l1_l11_id = _i(keep(dom.l1_l11_id, np.int32))
        d.l11_area_km2 = _d(keep(dom.l11_area_km2))
        d.l11_l1_id = _i(keep(dom.l11_l1_id, np.int32))
        d.net_perm = _i(keep(dom.net_perm, np.int32))
        d.from_n = _i(keep(dom.from_n, np.int32))
        d.to_n = _i(keep(dom.to_n, np.int32))
        d.length = _d(keep(dom.length))
        d.slope = _d(keep(dom.slope))
        d.ffp_imp = _d(keep(dom.ffp_imp))
        d.gauge_node = _i(keep(dom.gauge_node, np.int32))
        d.latitude = _d(keep(dom.latitude))
        self._desc = d
        ctx = C.c_void_p()
        rc = self.L.mhm_ctx_create(C.byref(d), device, C.byref(ctx))
        if rc != 0:
            raise MhmError(f"mhm_ctx_create failed ({rc})")
        self.ctx = ctx
        self._forcing_keep: dict[int, object] = {}

    # ---- lifetime ----
    def close(self):
        if getattr(self, "ctx", None):
            self.L.mhm_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.L.mhm_last_error(self.ctx).decode(errors="replace")
            raise MhmError(f"{what} failed ({rc}): {msg}")

    # ---- set-up (mhm_interface_run_prepare) ----
    def set_eff_params(self, p: dict[str, np.ndarray], member: int = 0):
        ep = _lib.EffParams()
        hold = []
        for name in _lib.EFF_PARAM_FIELDS:
            a = p.get(name)
            if a is not None:
                a = np.ascontiguousarray(a, np.float64)
                hold.append(a)
                setattr(ep, name, _d(a))
        self._check(self.L.mhm_set_eff_params(self.ctx, member, C.byref(ep)), "mhm_set_eff_params")

    def set_routing_params(self, p5, member: int = 0):
        a = np.ascontiguousarray(p5, np.float64)
        self._check(self.L.mhm_set_routing_params(self.ctx, member, _d(a)), "mhm_set_routing_params")

    def set_link_celerity(self, celerity, member: int = 0):
        """Routing case 3: each link's celerity [m s-1] (routing.link_celerity)."""
        a = np.ascontiguousarray(celerity, np.float64)
        self._check(self.L.mhm_set_link_celerity(self.ctx, member, _d(a)), "mhm_set_link_celerity")

    def set_meteo_weights(self, pre=None, pet=None, temp=None):
        """read_meteo_weights: hourly weights [24][12][n_cells] (the reference's
        L1_*_weights(cell, month, hour)) for pre, pet and temp; all None returns
        to the day/night ratios."""
        if pre is None and pet is None and temp is None:
            self._check(self.L.mhm_set_meteo_weights(self.ctx, None, None, None), "mhm_set_meteo_weights")
            return
        w = [np.ascontiguousarray(a, np.float64) for a in (pre, pet, temp)]
        self._check(self.L.mhm_set_meteo_weights(self.ctx, *[_d(a) for a in w]), "mhm_set_meteo_weights")

    def set_inflow_gauges(self, node, headwater, q=None, day0: int = 1):
        """Inflow gauges at the L11 nodes `node` (1-based) with headwater flags,
        and optionally their daily discharge q[days][gauges] [m3 s-1] from
        day0 (mhm_set_inflow_gauges / mhm_set_inflow_discharge)."""
        n = np.ascontiguousarray(node, np.int32)
        h = np.ascontiguousarray(np.asarray(headwater, bool).astype(np.int32))
        self._check(self.L.mhm_set_inflow_gauges(self.ctx, n.size, _i(n), _i(h)), "mhm_set_inflow_gauges")
        if q is not None:
            self.set_inflow_discharge(q, day0)

    def set_inflow_discharge(self, q, day0: int = 1):
        a = np.ascontiguousarray(q, np.float64)
        self._check(self.L.mhm_set_inflow_discharge(self.ctx, day0, a.shape[0], _d(a)), "mhm_set_inflow_discharge")

    def set_lai_series(self, mode: int, n_lai: int = 0):
        """timeStep_LAI_input: 0 monthly LAI slots (default); -1 / -2 / -3 a
        gridded LAI series of n_lai daily / monthly / yearly entries
        (mhm_set_lai_series)."""
        self._check(self.L.mhm_set_lai_series(self.ctx, int(mode), int(n_lai)), "mhm_set_lai_series")
        self._lai = (int(mode), int(n_lai)) if mode < 0 else (0, 12)

    def set_lai_params(self, max_inter, pet_lai=None, surf_resist=None, member: int = 0):
        """The member's LAI-indexed parameters of the series, each [n_lai][n_cells]."""
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (max_inter, pet_lai, surf_resist)]
        self._check(self.L.mhm_set_lai_params(self.ctx, member, *[_d(a) if a is not None else None for a in arrs]),
                    "mhm_set_lai_params")

    def get_lai_params(self, n_lai: int, member: int = 0) -> tuple:
        """(maxInter, pet group, surfResist) of the member's series, each [n_lai][n_cells]."""
        out = tuple(np.zeros((n_lai, self.dom.n_cells)) for _ in range(3))
        self._check(self.L.mhm_get_lai_params(self.ctx, member, *[_d(a) for a in out]), "mhm_get_lai_params")
        return out

    def set_link_fpimp(self, ffp):
        """Floodplain impervious fraction of the links for a new land-cover scene."""
        a = np.ascontiguousarray(ffp, np.float64)
        self._check(self.L.mhm_set_link_fpimp(self.ctx, _d(a)), "mhm_set_link_fpimp")

    def init_states(self, member: int = 0):
        hd = np.ascontiguousarray(self.dom.horizon_depth, np.float64)
        self._check(self.L.mhm_init_states(self.ctx, member, _d(hd)), "mhm_init_states")

    def prepare(self, params: dict[str, np.ndarray] | list, routing_params=None):
        """Effective parameters (one dict, or one per member), default states
        and Muskingum coefficients for every member."""
        plist = params if isinstance(params, list) else [params] * self.n_members
        rlist = routing_params if (routing_params is not None and np.ndim(routing_params) == 2) else \
            [routing_params] * self.n_members
        for m in range(self.n_members):
            self.set_eff_params(plist[m], m)
            self.init_states(m)
            if rlist[m] is not None:
                self.set_routing_params(rlist[m], m)

    def get_eff_params(self, member: int = 0) -> dict[str, np.ndarray]:
        """The member's effective parameters (L1_* arrays) read back."""
        N, H = self.dom.n_cells, self.dom.n_horizons
        sizes = {"maxInter": 12 * N, "petLAIcorFactor": 12 * N, "fRoots": H * N, "soilMoistSat": H * N,
                 "soilMoistFC": H * N, "wiltingPoint": H * N, "soilMoistExp": H * N, "PrieTayAlpha": 12 * N,
                 "aeroResist": 12 * N, "surfResist": 12 * N}
        out = {n: np.zeros(sizes.get(n, N)) for n in _lib.EFF_PARAM_FIELDS}
        ep = _lib.EffParams(**{n: _d(a) for n, a in out.items()})
        self._check(self.L.mhm_get_eff_params(self.ctx, member, C.byref(ep)), "mhm_get_eff_params")
        return out

    # ---- parameter regionalisation (mpr_eval) ----
    def mpr_setup(self, l0):
        """Level-0 maps and soil database of the basin (mhm_l0_desc from a
        synth.L0Maps)."""
        hold = []

        def k(a, dt=np.float64):
            a = np.ascontiguousarray(a, dt)
            hold.append(a)
            return a

        d = _lib.L0Desc()
        d.n_cells0, d.nrows0, d.ncols0 = l0.n_cells0, l0.nrows0, l0.ncols0
        d.n_soil_types, d.max_soil_hor, d.n_geo_units = l0.n_soil, l0.max_hor, l0.n_geo
        gridded = getattr(l0, "gridded_lai", False)
        d.n_lai_classes = 0 if gridded else int(l0.lai_lut.shape[0])
        d.frac_sealed_city = l0.frac_sealed_city
        d.horizon_depth = _d(k(l0.horizon_depth))
        d.mask0 = k(l0.mask0, np.uint8).ctypes.data_as(C.POINTER(C.c_uint8))
        for n in ("l1_up", "l1_down", "l1_left", "l1_right", "l1_nsub", "soil_id0", "lcover0", "geo_unit0",
                  "soil_n_hor", "soil_n_till", "geo_unit_list", "geo_unit_kar"):
            setattr(d, n, _i(k(getattr(l0, n), np.int32)))
        for n in ("slope0", "aspect0", "y0", "soil_ud", "soil_ld", "soil_sand", "soil_clay", "soil_dbm",
                  "soil_rz_depth"):
            setattr(d, n, _d(k(getattr(l0, n))))
        if gridded:
            lai0 = k(l0.lai0())
            d.lai0 = _d(lai0)
            d.n_lai_steps = int(lai0.shape[0])
        else:
            d.lai_class0 = _i(k(l0.lai_class0, np.int32))
            d.lai_lut = _d(k(l0.lai_lut))
        self._check(self.L.mhm_mpr_setup(self.ctx, C.byref(d)), "mhm_mpr_setup")
        self._l0 = l0

    def mpr(self, gammas: np.ndarray, member0: int = 0):
        """mpr() (and reg_rout) for members member0.. from global parameter
        vectors [n][n_gamma] (or one vector)."""
        g = np.ascontiguousarray(np.atleast_2d(gammas), np.float64)
        self._check(self.L.mhm_mpr(self.ctx, member0, g.shape[0], _d(g), g.shape[1]), "mhm_mpr")

    def mpr_aux(self, name: str) -> np.ndarray:
        l0 = self._l0
        size = {"Wd": l0.n_soil * self.dom.n_horizons * l0.max_hor, "slope_emp": l0.n_cells0,
                "horizon_depth": self.dom.n_horizons}[name]
        out = np.zeros(size)
        self._check(self.L.mhm_mpr_get_aux(self.ctx, name.encode(), _d(out)), "mhm_mpr_get_aux")
        return out

    # ---- forcing (set_meteo) ----
    def set_forcing(self, kind: int, row0: int, data, on_device: bool = False):
        """data: numpy [rows, N] (host) or an object with data_ptr() (device)."""
        if on_device:
            ptr = C.c_void_p(data.data_ptr())
            n_rows = int(data.shape[0])
        else:
            data = np.ascontiguousarray(data, np.float64)
            ptr = data.ctypes.data_as(C.c_void_p)
            n_rows = data.shape[0]
        self._forcing_keep[kind] = data
        self._check(self.L.mhm_set_forcing(self.ctx, kind, row0, n_rows, ptr, 1 if on_device else 0),
                    "mhm_set_forcing")

    def set_meteo(self, row0: int, pre, temp, pet=None, tmin=None, tmax=None, on_device: bool = False,
                  netrad=None, eabs=None, windspeed=None):
        self.set_forcing(_lib.FORC_PRE, row0, pre, on_device)
        self.set_forcing(_lib.FORC_TEMP, row0, temp, on_device)
        if pet is not None:
            self.set_forcing(_lib.FORC_PET, row0, pet, on_device)
        if tmin is not None:
            self.set_forcing(_lib.FORC_TMIN, row0, tmin, on_device)
        if tmax is not None:
            self.set_forcing(_lib.FORC_TMAX, row0, tmax, on_device)
        if netrad is not None:
            self.set_forcing(_lib.FORC_NETRAD, row0, netrad, on_device)
        if eabs is not None:
            self.set_forcing(_lib.FORC_EABS, row0, eabs, on_device)
        if windspeed is not None:
            self.set_forcing(_lib.FORC_WINDSPEED, row0, windspeed, on_device)

    # ---- time stepping (do_time_step x n) ----
    def enable_outputs(self, total_runoff: bool = False, qmod: bool = False):
        self._check(self.L.mhm_enable_outputs(self.ctx, int(total_runoff), int(qmod)), "mhm_enable_outputs")
        self._out = (total_runoff, qmod)

    def run(self, tt0: int, n_steps: int) -> np.ndarray:
        """Advance steps tt0..tt0+n_steps-1; returns gauge discharge
        [member, gauge, step] in m3 s-1."""
        G = len(self.dom.gauge_node)
        q = np.zeros((self.n_members, G, n_steps), np.float64)
        self._check(self.L.mhm_run(self.ctx, tt0, n_steps, _d(q) if G else None), "mhm_run")
        self._last_steps = n_steps
        return q

    def run_async(self, tt0: int, n_steps: int, q_out: np.ndarray | None = None):
        """Enqueue steps tt0..tt0+n_steps-1 and return at once; q_out
        ([member, gauge, step] float64, kept alive by the caller) is filled
        when sync() returns."""
        self._check(self.L.mhm_run_async(self.ctx, tt0, n_steps, _d(q_out) if q_out is not None else None),
                    "mhm_run_async")
        self._last_steps = n_steps

    def run_members_async(self, member_tt0, n_steps: int, q_out: np.ndarray | None = None):
        """Enqueue n_steps for every member from its own step member_tt0[m]
        (<= 0: idle); forcing = rows 0..n_steps-1 of the device window."""
        t0 = np.ascontiguousarray(member_tt0, np.int32)
        self._t0_keep = t0
        self._check(self.L.mhm_run_members_async(self.ctx, _i(t0), n_steps, _d(q_out) if q_out is not None else None),
                    "mhm_run_members_async")
        self._last_steps = n_steps

    def enable_fluxes(self, on: bool = True):
        self._check(self.L.mhm_enable_fluxes(self.ctx, 1 if on else 0), "mhm_enable_fluxes")
        self._fluxes = on

    def get_fluxes(self) -> tuple[np.ndarray, np.ndarray]:
        """(aET, karst loss) of the last run, each [step, member, cell]."""
        n = self._last_steps
        aet = np.zeros((n, self.n_members, self.dom.n_cells))
        loss = np.zeros_like(aet)
        self._check(self.L.mhm_get_fluxes(self.ctx, _d(aet), _d(loss)), "mhm_get_fluxes")
        return aet, loss

    def enable_flux_state_outputs(self, flags, interval: int, warming_steps: int, n_time_steps: int,
                                  max_slots: int = 32):
        """Aggregated per-cell outputs (outputFlxState flags: 21 ints, or indexes /
        names for outputs.flags_from) closed at timeStep_model_outputs `interval`."""
        flags = list(flags) if len(flags) == 21 and all(f in (0, 1) for f in flags) else outputs.flags_from(flags)
        cfg = _lib.OutputConfig(timestep_model_outputs=interval, max_slots=max_slots, warming_steps=warming_steps,
                                n_time_steps=n_time_steps)
        for i, f in enumerate(flags):
            cfg.flags[i] = int(f)
        self._check(self.L.mhm_enable_flux_state_outputs(self.ctx, C.byref(cfg)), "mhm_enable_flux_state_outputs")
        self._fs_names = outputs.plane_names(flags, self.dom.n_horizons)
        self._fs_slots = max_slots

    def read_flux_state_outputs(self) -> tuple[list[str], np.ndarray, np.ndarray]:
        """(plane names, closed intervals [slot][plane][member][cell], the model
        step closing each slot); frees the device slots."""
        n = C.c_int32()
        npl = C.c_int32()
        self._check(self.L.mhm_read_flux_state_outputs(self.ctx, None, None, 0, C.byref(n), C.byref(npl)),
                    "mhm_read_flux_state_outputs")
        out = np.zeros((n.value, npl.value, self.n_members, self.dom.n_cells))
        tt = np.zeros(max(n.value, 1), np.int64)
        self._check(self.L.mhm_read_flux_state_outputs(self.ctx, _d(out), tt.ctypes.data_as(C.POINTER(C.c_int64)),
                                                       n.value, C.byref(n), C.byref(npl)),
                    "mhm_read_flux_state_outputs")
        return self._fs_names, out, tt[: n.value]

    def enable_routed_outputs(self, interval: int, warming_steps: int, n_time_steps: int, max_slots: int = 32):
        """mRM's Qrouted output (mean L11 discharge per interval)."""
        cfg = _lib.OutputConfig(timestep_model_outputs=interval, max_slots=max_slots, warming_steps=warming_steps,
                                n_time_steps=n_time_steps)
        cfg.flags[0] = 1
        self._check(self.L.mhm_enable_routed_outputs(self.ctx, C.byref(cfg)), "mhm_enable_routed_outputs")

    def read_routed_outputs(self) -> tuple[np.ndarray, np.ndarray]:
        """(Qrouted [slot][member][node] in L11 node order, closing steps)."""
        n = C.c_int32()
        self._check(self.L.mhm_read_routed_outputs(self.ctx, None, None, 0, C.byref(n)), "mhm_read_routed_outputs")
        out = np.zeros((n.value, self.n_members, self.dom.n_nodes))
        tt = np.zeros(max(n.value, 1), np.int64)
        self._check(self.L.mhm_read_routed_outputs(self.ctx, _d(out), tt.ctypes.data_as(C.POINTER(C.c_int64)),
                                                   n.value, C.byref(n)), "mhm_read_routed_outputs")
        return out, tt[: n.value]

    def set_output_weights(self, member: int, tt: int, fsealed=None, soil_moist_sat=None):
        """Outputs of step tt weighted with these fSealed [cell] / soilMoistSat
        [horizon][cell] (the next land-cover scene's); tt < 1 clears."""
        fs = None if fsealed is None else np.ascontiguousarray(fsealed, np.float64)
        sm = None if soil_moist_sat is None else np.ascontiguousarray(soil_moist_sat, np.float64)
        self._check(self.L.mhm_set_output_weights(self.ctx, member, tt, _d(fs), _d(sm)), "mhm_set_output_weights")

    def autotune(self, tt0: int, n_steps: int, route: bool = True) -> dict:
        """Pick the fastest cell-chain register variant and routing sub-chunk
        by timing n_steps from tt0 (states restored afterwards), then, with
        `route`, the routing launch mode (per-tick graph or cluster walk)."""
        occ = C.c_int32()
        sub = C.c_int32()
        ms = np.zeros(9)
        self._check(self.L.mhm_autotune(self.ctx, tt0, n_steps, C.byref(occ), C.byref(sub), _d(ms)), "mhm_autotune")
        out = {"cell_blocks_per_sm": occ.value, "route_sub_steps": sub.value, "trial_ms": ms.tolist()}
        if route:
            out.update(self.autotune_route(tt0, n_steps))
        return out

    def autotune_route(self, tt0: int, n_steps: int) -> dict:
        """mhm_autotune_route: route_cluster 0 (per-tick graph), 4, 8, 16 timed;
        the fastest is kept."""
        cl = C.c_int32()
        ms = np.zeros(4)
        self._check(self.L.mhm_autotune_route(self.ctx, tt0, n_steps, C.byref(cl), _d(ms)), "mhm_autotune_route")
        return {"route_cluster": cl.value, "route_trial_ms": ms.tolist()}

    def autotune_ex(self, tt0: int, n_steps: int, chunk_choices=()) -> dict:
        """The autotuner over register variant x routing sub-chunk x time-chunk
        length (mhm_autotune_ex); returns the configuration kept."""
        ch = np.ascontiguousarray(chunk_choices, np.int32)
        nc = max(1, ch.size)
        ms = np.zeros(9 * nc)
        best = _lib.LaunchConfig()
        self._check(self.L.mhm_autotune_ex(self.ctx, tt0, n_steps, ch.size, _i(ch) if ch.size else None,
                                           C.byref(best), _d(ms)), "mhm_autotune_ex")
        return {"cell_blocks_per_sm": best.cell_blocks_per_sm, "route_sub_steps": best.route_sub_steps,
                "chunk_steps": best.chunk_steps, "route_cluster": best.route_cluster, "trial_ms": ms.tolist()}

    def set_launch_config(self, cell_blocks_per_sm: int = 4, route_sub_steps: int = 8, chunk_steps: int = 0,
                          route_cluster: int = 0):
        cfg = _lib.LaunchConfig(cell_blocks_per_sm, route_sub_steps, chunk_steps, route_cluster)
        self._check(self.L.mhm_set_launch_config(self.ctx, C.byref(cfg)), "mhm_set_launch_config")

    def get_launch_config(self) -> dict:
        cfg = _lib.LaunchConfig()
        self._check(self.L.mhm_get_launch_config(self.ctx, C.byref(cfg)), "mhm_get_launch_config")
        return {"cell_blocks_per_sm": cfg.cell_blocks_per_sm, "route_sub_steps": cfg.route_sub_steps,
                "chunk_steps": cfg.chunk_steps, "route_cluster": cfg.route_cluster}

    def snapshot_alloc(self, n_slots: int):
        self._check(self.L.mhm_snapshot_alloc(self.ctx, n_slots), "mhm_snapshot_alloc")

    def snapshot_save(self, member: int, slot: int):
        self._check(self.L.mhm_snapshot_save(self.ctx, member, slot), "mhm_snapshot_save")

    def snapshot_load(self, slot: int, member: int):
        self._check(self.L.mhm_snapshot_load(self.ctx, slot, member), "mhm_snapshot_load")

    def member_status(self) -> np.ndarray:
        """Per-member status since the last call (mhm_member_status): 0, or
        MHM_ERR_NAN for a member whose states or runoff became non-finite."""
        st = np.zeros(self.n_members, np.int32)
        rc = self.L.mhm_member_status(self.ctx, _i(st))
        if rc not in (0, _lib.MHM_ERR_NAN):
            self._check(rc, "mhm_member_status")
        return st

    def sync(self):
        self._check(self.L.mhm_sync(self.ctx), "mhm_sync")

    def device_status(self):
        """None, or (site, index) of the first failed index test of the
        bounds-checked build (mhm_device_status; clears it)."""
        site = C.c_int32()
        idx = C.c_int64()
        rc = self.L.mhm_device_status(self.ctx, C.byref(site), C.byref(idx))
        if rc == _lib.MHM_ERR_BOUNDS:
            return int(site.value), int(idx.value)
        self._check(rc, "mhm_device_status")
        return None

    def bounds_selftest(self):
        self._check(self.L.mhm_bounds_selftest(self.ctx), "mhm_bounds_selftest")

    def poll(self) -> bool:
        """True if all enqueued work has completed (sync() then returns at once)."""
        d = C.c_int32()
        self._check(self.L.mhm_poll(self.ctx, C.byref(d)), "mhm_poll")
        return bool(d.value)

    def get_outputs(self):
        n = self._last_steps
        tro = np.zeros((n, self.n_members, self.dom.n_cells)) if self._out[0] else None
        qm = np.zeros((self.n_members, n, self.dom.n_nodes)) if self._out[1] else None
        self._check(self.L.mhm_get_outputs(self.ctx, _d(tro), _d(qm)), "mhm_get_outputs")
        return tro, qm

    # ---- state access (restart fields, get_variable) ----
    def get_state(self, member: int = 0) -> dict[str, np.ndarray]:
        N, H, L = self.dom.n_cells, self.dom.n_horizons, self.dom.n_nodes
        shapes = {"interc": N, "snowpack": N, "sealSTW": N, "unsatSTW": N, "satSTW": N,
                  "soilMoist": H * N, "qOUT": L, "Qmod": L, "qTIN": 2 * L, "qTR": 2 * L, "C1": L, "C2": L}
        out = {k: np.zeros(v) for k, v in shapes.items()}
        st = _lib.Restart(**{k: _d(v) for k, v in out.items()})
        self._check(self.L.mhm_get_state(self.ctx, member, C.byref(st)), "mhm_get_state")
        return out

    def set_state(self, state: dict[str, np.ndarray], member: int = 0):
        arrs = {k: np.ascontiguousarray(v, np.float64) for k, v in state.items()}
        st = _lib.Restart(**{k: _d(v) for k, v in arrs.items()})
        self._check(self.L.mhm_set_state(self.ctx, member, C.byref(st)), "mhm_set_state")

    def load_restart(self, mhm, scene: int = 0, mrm=None, member: int = 0):
        """Start from restart files (read_restart = .true.): the land-cover
        scene's effective parameters and the L1 states of an mHM restart
        (restart.MhmRestart), with an mRM restart (restart.MrmRestart) also
        the routing states and Muskingum coefficients -- no MPR, no soil
        moisture initialisation (src/mHM/mo_mhm_interface_run.f90:221-236).
        Create the context with read_states=True so that step 1 keeps them."""
        if int(mhm.mask.sum()) != self.dom.n_cells:
            raise MhmError(f"restart has {int(mhm.mask.sum())} L1 cells, the domain {self.dom.n_cells}")
        p = mhm.eff_params(scene)
        n_lai = mhm.n_lai
        if self._lai[0] < 0 or n_lai != 12:
            # a gridded LAI series: its entries go to the context's series
            if self._lai[0] >= 0 or self._lai[1] != n_lai:
                raise MhmError(f"the restart holds {n_lai} LAI entries: set_lai_series(mode, {n_lai}) first")
            lp = mhm.lai_params(scene)
            pet = {-1: "petLAIcorFactor", 2: "PrieTayAlpha", 3: "aeroResist"}.get(self.proc_pet)
            self.set_lai_params(lp["maxInter"], lp.get(pet) if pet else None, lp.get("surfResist"), member)
            N = self.dom.n_cells
            for k in ("maxInter", "petLAIcorFactor", "PrieTayAlpha", "aeroResist", "surfResist"):
                if k in p:
                    p[k] = np.resize(p[k], 12 * N)   # the monthly slots are not read with a series
        self.set_eff_params(p, member)
        st = dict(mhm.states)
        if mrm is not None:
            if int(mrm.mask.sum()) != self.dom.n_nodes:
                raise MhmError(f"restart has {int(mrm.mask.sum())} L11 nodes, the domain {self.dom.n_nodes}")
            st.update(mrm.states)
        self.set_state(st, member)

    def write_restart(self, mhm_path, params_by_scene: list[dict], mask=None, mrm_path=None, mask11=None,
                      network: dict | None = None, member: int = 0):
        """Write the member's states (and the given scenes' effective
        parameters) as an mHM restart, and its routing states as an mRM
        restart, in the reference's layout.  mask / mask11: the L1 / L11 grids
        ([ncols][nrows] bool, default one row of all cells)."""
        from . import restart
        st = self.get_state(member)
        m1 = np.ones((1, self.dom.n_cells), bool) if mask is None else np.asarray(mask, bool)
        restart.write_mhm_restart(mhm_path, m1, st, params_by_scene, self.dom.horizon_depth,
                                  proc_sm=self.proc_soilmoist, proc_pet=self.proc_pet)
        if mrm_path is not None:
            m11 = np.ones((1, self.dom.n_nodes), bool) if mask11 is None else np.asarray(mask11, bool)
            restart.write_mrm_restart(mrm_path, m11, {k: st[k] for k in restart.MRM_STATES.values()},
                                      network or {}, mask1=m1)

    def get_variable(self, name: str, member: int = 0) -> np.ndarray:
        n = {"L1_SOILMOIST": self.dom.n_horizons * self.dom.n_cells, "L11_QMOD": self.dom.n_nodes,
             "L11_QOUT": self.dom.n_nodes}.get(name, self.dom.n_cells)
        out = np.zeros(n)
        self._check(self.L.mhm_get_var(self.ctx, member, name.encode(), _d(out)), "mhm_get_var")
        return out

    # ---- timing ----
    def set_timing(self, on: bool):
        self._check(self.L.mhm_set_timing(self.ctx, int(on)), "mhm_set_timing")

    def get_timing(self, kind: int) -> tuple[int, float]:
        n = C.c_int64()
        ms = C.c_double()
        self._check(self.L.mhm_get_timing(self.ctx, kind, C.byref(n), C.byref(ms)), "mhm_get_timing")
        return n.value, ms.value

    @property
    def stream(self) -> int:
        return int(self.L.mhm_ctx_stream(self.ctx) or 0)


class MhmBatch:
    """Contexts whose cell chains run in one persistent launch per call
    (mhm_batch_run_members): each call enqueues one chunk of per-member
    steps on every context given, as MhmGpu.run_members_async would."""

    def __init__(self, device: int = -1):
        self.L = _lib.load()
        b = C.c_void_p()
        rc = self.L.mhm_batch_create(device, C.byref(b))
        if rc != 0:
            raise MhmError(f"mhm_batch_create failed ({rc})")
        self.b = b

    def run_members(self, ctxs: list, member_tt0s: list, n_steps: int, q_outs: list | None = None):
        n = len(ctxs)
        vp = C.c_void_p
        cs = (vp * n)(*[g.ctx.value for g in ctxs])
        t0s = [np.ascontiguousarray(t, np.int32) for t in member_tt0s]
        tp = (C.POINTER(C.c_int32) * n)(*[_i(t) for t in t0s])
        qp = None
        if q_outs is not None:
            qp = (C.POINTER(C.c_double) * n)(*[_d(q) if q is not None else None for q in q_outs])
        for g, t in zip(ctxs, t0s):
            g._t0_keep = t
            g._last_steps = n_steps
        rc = self.L.mhm_batch_run_members(self.b, n, cs, tp, n_steps, qp)
        if rc != 0:
            raise MhmError(f"mhm_batch_run_members failed ({rc}): "
                           f"{self.L.mhm_batch_last_error(self.b).decode(errors='replace')}")

    def close(self):
        if getattr(self, "b", None):
            self.L.mhm_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
