"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py -- never by the mhm_gb300 package.  `build()` compiles both variants
(hmath and libm elementary functions) with the Makefile next to this file.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


def build() -> None:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


class OraDomain(C.Structure):
    _fields_ = [
        ("nCells", C.c_int32), ("nH", C.c_int32), ("nNodes", C.c_int32), ("nOutlets", C.c_int32),
        ("timestep", C.c_int32), ("proc_sm", C.c_int32), ("proc_pet", C.c_int32), ("proc_rout", C.c_int32),
        ("nTstepForcingDay", C.c_int32), ("read_states", C.c_int32), ("jul_start", C.c_int32),
        ("map_flag", C.c_int32), ("nGauges", C.c_int32), ("pad_", C.c_int32),
        ("evap_coeff", _dp), ("fday_prec", _dp), ("fnight_prec", _dp), ("fday_pet", _dp),
        ("fnight_pet", _dp), ("fday_temp", _dp), ("fnight_temp", _dp),
        ("l1_area_km2", _dp), ("l1_l11_id", _ip), ("l11_area_km2", _dp), ("l11_l1_id", _ip),
        ("net_perm", _ip), ("from_n", _ip), ("to_n", _ip), ("length", _dp), ("slope", _dp),
        ("ffp_imp", _dp), ("rout_param", _dp), ("gauge_node", _ip), ("latitude", _dp), ("link_celerity", _dp),
        ("pre_w", _dp), ("pet_w", _dp), ("temp_w", _dp),
        ("nInflow", C.c_int32), ("inflow_day0", C.c_int32), ("inflow_ndays", C.c_int32), ("pad2_", C.c_int32),
        ("inflow_node", _ip), ("inflow_headwater", _ip), ("inflow_q", _dp),
        ("lai_mode", C.c_int32), ("n_lai", C.c_int32),
    ]


PARAM_FIELDS = ["fSealed", "alpha", "degDayInc", "degDayMax", "degDayNoPre", "fAsp", "HarSamCoeff",
                "karstLoss", "kFastFlow", "kSlowFlow", "kBaseFlow", "kPerco", "jarvis_c1", "tempThresh",
                "unsatThresh", "sealedThresh", "maxInter", "petLAIcorFactor", "fRoots", "SMs", "FC", "PW",
                "beta", "PrieTayAlpha", "aeroResist", "surfResist"]
# mhm_eff_params name -> oracle name
PARAM_ALIAS = {"jarvis_thresh_c1": "jarvis_c1", "soilMoistSat": "SMs", "soilMoistFC": "FC",
               "wiltingPoint": "PW", "soilMoistExp": "beta"}


class OraParams(C.Structure):
    _fields_ = [(n, _dp) for n in PARAM_FIELDS]


STATE_FIELDS = ["interc", "snowpack", "sealSTW", "SM", "unsat", "sat", "qTIN", "qTR", "qOUT", "Qmod", "C1", "C2",
                "run_to_rout"]


class OraState(C.Structure):
    _fields_ = [(n, _dp) for n in STATE_FIELDS]


class OraForcing(C.Structure):
    _fields_ = [("pre", _dp), ("temp", _dp), ("pet", _dp), ("tmin", _dp), ("tmax", _dp),
                ("forc_row0", C.c_int32), ("n_rows", C.c_int32), ("netrad", _dp), ("eabs", _dp),
                ("windspeed", _dp)]


class OraOutput(C.Structure):
    _fields_ = [
        ("interval", C.c_int32), ("interval_mrm", C.c_int32), ("warm_steps", C.c_int32),
        ("n_time_steps", C.c_int32), ("flags", C.c_int32 * 21), ("qrouted", C.c_int32), ("max_slots", C.c_int32),
        ("n_planes", C.c_int32), ("plane", C.c_int32 * 22), ("counter", C.c_int32), ("counter_mrm", C.c_int32),
        ("n_slots", C.c_int32), ("n_slots_mrm", C.c_int32), ("tt_w", C.c_int32), ("pad_", C.c_int32),
        ("acc", _dp), ("out", _dp), ("slot_tt", _ip), ("acc_mrm", _dp), ("out_mrm", _dp), ("slot_tt_mrm", _ip),
        ("w_fsealed", _dp), ("w_sms", _dp),
    ]


class OraMprDomain(C.Structure):
    _fields_ = [
        ("nCells0", C.c_int32), ("nrows0", C.c_int32), ("ncols0", C.c_int32), ("nCells1", C.c_int32),
        ("nH", C.c_int32), ("nSoil", C.c_int32), ("maxHor", C.c_int32), ("nGeo", C.c_int32),
        ("proc_sm", C.c_int32), ("proc_pet", C.c_int32), ("n_soil_params", C.c_int32), ("nLAI", C.c_int32),
        ("fracSealed_cityArea", C.c_double), ("id0_2d", _ip),
        ("up1", _ip), ("down1", _ip), ("left1", _ip), ("right1", _ip), ("nsub1", _ip),
        ("LCover0", _ip), ("soilId0", _ip), ("geoUnit0", _ip), ("slope_emp0", _dp), ("Asp0", _dp), ("y0", _dp),
        ("LAI0", _dp), ("present", _ip), ("nHor", _ip), ("nTill", _ip), ("sand", _dp), ("clay", _dp),
        ("DbM", _dp), ("RZdepth", _dp), ("Wd", _dp), ("horizonDepth", _dp), ("geoUnitList", _ip),
        ("geoUnitKar", _ip),
    ]


class OraGamma(C.Structure):
    _fields_ = [(n, _dp) for n in ("interc", "snow", "soil", "runoff", "pet", "interflow", "perc", "geo")]


MPR_OUT_FIELDS = ["fSealed", "alpha", "degDayInc", "degDayMax", "degDayNoPre", "fAsp", "HarSamCoeff",
                  "karstLoss", "kFastFlow", "kSlowFlow", "kBaseFlow", "kPerco", "jarvis_c1", "tempThresh",
                  "unsatThresh", "sealedThresh", "maxInter", "petLAIcorFactor", "fRoots", "SMs", "FC", "PW",
                  "beta", "PrieTayAlpha", "aeroResist", "surfResist"]


class OraMprOut(C.Structure):
    _fields_ = [(n, _dp) for n in MPR_OUT_FIELDS]


_LIBS: dict[str, C.CDLL] = {}


def load(kind: str = "hmath") -> C.CDLL:
    """kind: 'hmath' (the GPU's elementary functions) or 'libm' (the C library's)."""
    if kind in _LIBS:
        return _LIBS[kind]
    path = BUILD / f"liboracle_{kind}.so"
    if not path.exists():
        build()
    L = C.CDLL(str(path))
    d = C.c_double
    L.ora_canopy_interc.argtypes = [d, d, d, _dp, _dp, _dp]
    L.ora_snow_accum_melt.argtypes = [d, d, d, d, d, d, d, _dp, _dp, _dp, _dp, _dp, _dp]
    L.ora_feddes_et_reduction.argtypes = [d, d, d, d]
    L.ora_feddes_et_reduction.restype = d
    L.ora_jarvis_et_reduction.argtypes = [d, d, d, d, d]
    L.ora_jarvis_et_reduction.restype = d
    L.ora_soil_moisture.argtypes = [C.c_int, C.c_int, d, d, d, d, _dp, _dp, _dp, _dp, _dp, d, d, d,
                                    _dp, _dp, _dp, _dp, _dp, _dp]
    L.ora_runoff_unsat_zone.argtypes = [d, d, d, d, d, d, d, _dp, _dp, _dp, _dp, _dp]
    L.ora_runoff_sat_zone.argtypes = [d, _dp, _dp]
    L.ora_L1_total_runoff.argtypes = [d, d, d, d, d]
    L.ora_L1_total_runoff.restype = d
    L.ora_extraterr_rad_approx.argtypes = [C.c_int, d]
    L.ora_extraterr_rad_approx.restype = d
    L.ora_pet_hargreaves.argtypes = [d, d, d, d, d, d, C.c_int]
    L.ora_pet_hargreaves.restype = d
    for f in ("ora_sat_vap_pressure", "ora_slope_satpressure"):
        getattr(L, f).argtypes = [d]
        getattr(L, f).restype = d
    L.ora_pet_priestly.argtypes = [d, d, d]
    L.ora_pet_priestly.restype = d
    L.ora_pet_penman.argtypes = [d, d, d, d, d, d, d]
    L.ora_pet_penman.restype = d
    L.ora_disagg_meteo_weights.argtypes = [d, d, d]
    L.ora_disagg_meteo_weights.restype = d
    L.ora_disagg_flux_daynight.argtypes = [C.c_int, d, d, d, d]
    L.ora_disagg_flux_daynight.restype = d
    L.ora_disagg_state_daynight.argtypes = [C.c_int, d, d, d, d, C.c_int]
    L.ora_disagg_state_daynight.restype = d
    L.ora_julday.argtypes = [C.c_int32] * 3
    L.ora_julday.restype = C.c_int32
    L.ora_caldat.argtypes = [C.c_int32, _ip, _ip, _ip]
    L.ora_dec2date.argtypes = [d, _ip, _ip, _ip, _ip, _ip, _ip]
    L.ora_step_calendar.argtypes = [C.c_int32, C.c_int32, C.c_int32, _ip, _ip, _ip, _ip, _ip]
    L.ora_reg_rout.argtypes = [_dp, _dp, _dp, _dp, C.c_int, d, _dp, _dp]
    L.ora_L11_runoff_acc.argtypes = [C.c_int, C.c_int, _dp, _dp, _ip, _dp, _ip, C.c_int, C.c_int, _dp]
    L.ora_L11_routing.argtypes = [C.c_int, C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp]
    L.ora_L11_set_network_topology.argtypes = [C.c_int, C.c_int, _ip, C.c_int, _ip, _ip, _ip, _ip, _ip]
    L.ora_L11_set_network_topology.restype = C.c_int
    L.ora_L11_routing_order.argtypes = [C.c_int, C.c_int, _ip, _ip, _ip, _ip]
    L.ora_L11_routing_order_listed.argtypes = [C.c_int, C.c_int, _ip, _ip, _ip, _ip]
    L.ora_L11_routing_order_listed.restype = C.c_int
    L.ora_update_param_case2.argtypes = [d, _dp, C.c_int, _dp, _dp]
    L.ora_update_param_case2.restype = d
    L.ora_update_param_links.argtypes = [_dp, d, _dp, C.c_int, _dp, _dp]
    L.ora_update_param_links.restype = d
    L.ora_add_inflow.argtypes = [C.c_int, _ip, _ip, _dp, _dp]
    L.ora_link_celerity.argtypes = [d, _dp, C.c_int]
    L.ora_link_celerity.restype = d
    L.ora_run.argtypes = [C.POINTER(OraDomain), C.POINTER(OraParams), C.POINTER(OraState),
                          C.POINTER(OraForcing), C.c_int32, C.c_int32, _dp, _dp, _dp, C.c_int]
    L.ora_run_ex.argtypes = [C.POINTER(OraDomain), C.POINTER(OraParams), C.POINTER(OraState),
                             C.POINTER(OraForcing), C.c_int32, C.c_int32, _dp, _dp, _dp, C.c_int,
                             C.POINTER(OraOutput)]
    L.ora_output_planes.argtypes = [C.POINTER(OraOutput), C.c_int]
    L.ora_output_planes.restype = C.c_int
    L.ora_step_calendar_ex.argtypes = [C.c_int32, C.c_int32, C.c_int32, _ip, _ip, _ip, _ip, _ip, _ip]
    L.ora_step_lai.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, _ip]
    L.ora_default_states.argtypes = [C.POINTER(OraDomain), _dp, C.POINTER(OraState)]
    L.ora_math_kind.restype = C.c_int
    L.ora_mpr.argtypes = [C.POINTER(OraMprDomain), C.POINTER(OraGamma), C.POINTER(OraMprOut)]
    L.ora_mpr.restype = C.c_int
    L.ora_soil_weights.argtypes = [C.c_int, C.c_int, _ip, _dp, _dp, _dp, C.c_int, _dp, _dp]
    L.ora_soil_weights.restype = C.c_int
    L.ora_slope_emp.argtypes = [C.c_int, _dp, _dp]
    L.ora_slope_emp.restype = C.c_int
    _LIBS[kind] = L
    return L


def routing_order(from_n, to_n, n_nodes: int, n_outlets: int, kind: str = "libm"):
    """(netPerm, rOrder) of L11_routing_order by the oracle's listed sweep
    (the reference's ranks; no use of the GPU library)."""
    L = load(kind)
    perm = np.zeros(n_nodes, np.int32)
    rord = np.zeros(n_nodes, np.int32)
    fn = np.ascontiguousarray(from_n, np.int32)
    tn = np.ascontiguousarray(to_n, np.int32)
    rc = L.ora_L11_routing_order_listed(n_nodes, n_outlets, _i(fn), _i(tn), _i(perm), _i(rord))
    if rc != 0:
        raise RuntimeError("routing order: the network has a cycle")
    return perm, rord


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


class OracleRun:
    """The mhm_eval time loop of one basin on the CPU (oracle)."""

    def __init__(self, dom, params: dict, rout_param=None, proc_sm=1, proc_pet=0, proc_rout=1,
                 hourly=True, read_states=False, kind="hmath", link_celerity=None, meteo_weights=None,
                 inflow=None, lai_mode: int = 0, n_lai: int = 12):
        self.L = load(kind)
        self.dom = dom
        self.keep = []

        def k(a, dt=np.float64):
            a = np.ascontiguousarray(a, dt)
            self.keep.append(a)
            return a

        d = OraDomain()
        d.nCells, d.nH, d.nNodes, d.nOutlets = dom.n_cells, dom.n_horizons, dom.n_nodes, dom.n_outlets
        d.timestep, d.proc_sm, d.proc_pet, d.proc_rout = dom.timestep, proc_sm, proc_pet, proc_rout
        d.nTstepForcingDay = 24 if hourly else 1
        d.read_states = int(read_states)
        d.jul_start = dom.jul_start
        d.map_flag = 1
        d.nGauges = len(dom.gauge_node)
        for n in ("evap_coeff", "fday_prec", "fnight_prec", "fday_pet", "fnight_pet", "fday_temp", "fnight_temp",
                  "l11_area_km2", "length", "slope", "ffp_imp", "latitude", "l1_area_km2"):
            setattr(d, n, _d(k(getattr(dom, n))))
        for n in ("l1_l11_id", "l11_l1_id", "net_perm", "from_n", "to_n", "gauge_node"):
            setattr(d, n, _i(k(getattr(dom, n), np.int32)))
        rp = k(np.resize(np.asarray(rout_param if rout_param is not None else np.zeros(5), np.float64), 5))
        d.rout_param = _d(rp)
        if link_celerity is not None:
            d.link_celerity = _d(k(link_celerity))
        if inflow is not None:   # {"node": [G] 1-based L11 ids, "headwater": [G], "day0": d, "q": [days][G]}
            d.nInflow = len(inflow["node"])
            d.inflow_node = _i(k(inflow["node"], np.int32))
            d.inflow_headwater = _i(k(inflow["headwater"], np.int32))
            q = k(inflow["q"])
            d.inflow_day0 = int(inflow.get("day0", 1))
            d.inflow_ndays = q.shape[0]
            d.inflow_q = _d(q)
        # timeStep_LAI_input: 0 = monthly slots; -1 / -2 / -3 = a gridded LAI series of
        # n_lai daily / monthly / yearly entries (the LAI-indexed parameters then have
        # n_lai entries per cell)
        d.lai_mode, d.n_lai = int(lai_mode), int(n_lai)
        if meteo_weights is not None:   # {"pre", "pet", "temp"}: [24][12][n_cells] each
            for n in ("pre", "pet", "temp"):
                setattr(d, n + "_w", _d(k(meteo_weights[n])))
        self.d = d
        p = OraParams()
        for name, arr in params.items():
            oname = PARAM_ALIAS.get(name, name)
            if oname in PARAM_FIELDS and arr is not None:
                setattr(p, oname, _d(k(arr)))
        self.p = p
        N, H, Ln = dom.n_cells, dom.n_horizons, dom.n_nodes
        self.state = {"interc": np.zeros(N), "snowpack": np.zeros(N), "sealSTW": np.zeros(N),
                      "SM": np.zeros(H * N), "unsat": np.zeros(N), "sat": np.zeros(N),
                      "qTIN": np.zeros(2 * Ln), "qTR": np.zeros(2 * Ln), "qOUT": np.zeros(Ln),
                      "Qmod": np.zeros(Ln), "C1": np.zeros(Ln), "C2": np.zeros(Ln), "run_to_rout": np.zeros(N)}
        self.s = OraState(**{n: _d(self.state[n]) for n in STATE_FIELDS})
        hd = k(dom.horizon_depth)
        self.L.ora_default_states(C.byref(self.d), _d(hd), C.byref(self.s))

    def enable_outputs(self, interval: int, flags, warm_steps: int, n_time_steps: int, max_slots: int,
                       interval_mrm: int | None = None, qrouted: bool = False):
        """Aggregated outputs of the following runs: flags = outputFlxState(1..21)
        (21 ints); Qrouted with `qrouted` at `interval_mrm`."""
        o = OraOutput()
        o.interval = interval
        o.interval_mrm = interval if interval_mrm is None else interval_mrm
        o.warm_steps, o.n_time_steps, o.max_slots = warm_steps, n_time_steps, max_slots
        for i, f in enumerate(flags):
            o.flags[i] = int(bool(f))
        o.qrouted = int(qrouted)
        N, H, Ln = self.dom.n_cells, self.dom.n_horizons, self.dom.n_nodes
        n = self.L.ora_output_planes(C.byref(o), H)
        if n < 0:
            raise ValueError("unsupported output variable")
        self.out_buf = {"acc": np.zeros(max(n, 1) * N), "out": np.zeros(max_slots * max(n, 1) * N),
                        "slot_tt": np.zeros(max_slots, np.int32), "acc_mrm": np.zeros(Ln),
                        "out_mrm": np.zeros(max_slots * Ln), "slot_tt_mrm": np.zeros(max_slots, np.int32)}
        for k in ("acc", "out", "acc_mrm", "out_mrm"):
            setattr(o, k, _d(self.out_buf[k]))
        o.slot_tt, o.slot_tt_mrm = _i(self.out_buf["slot_tt"]), _i(self.out_buf["slot_tt_mrm"])
        self.out = o

    def set_output_weights(self, tt: int, fsealed, soil_moist_sat):
        """Outputs of step tt weighted with these fSealed / soilMoistSat."""
        self.out_w = (np.ascontiguousarray(fsealed, np.float64), np.ascontiguousarray(soil_moist_sat, np.float64))
        self.out.tt_w = tt
        self.out.w_fsealed, self.out.w_sms = _d(self.out_w[0]), _d(self.out_w[1])

    def read_outputs(self):
        """(fluxes/states [slots][planes][cells], their closing steps, Qrouted
        [slots][nodes], its closing steps); frees the slots."""
        o, b = self.out, self.out_buf
        N, Ln = self.dom.n_cells, self.dom.n_nodes
        n = o.n_planes
        fs = b["out"][: o.n_slots * n * N].reshape(o.n_slots, n, N).copy()
        qr = b["out_mrm"][: o.n_slots_mrm * Ln].reshape(o.n_slots_mrm, Ln).copy()
        r = (fs, b["slot_tt"][: o.n_slots].copy(), qr, b["slot_tt_mrm"][: o.n_slots_mrm].copy())
        o.n_slots = o.n_slots_mrm = 0
        return r

    def run(self, forcing: dict, row0: int, tt0: int, n_steps: int, nthreads: int = 0,
            want_tro: bool = False, want_qmod: bool = False):
        f = OraForcing()
        keep = []
        for n in ("pre", "temp", "pet", "tmin", "tmax", "netrad", "eabs", "windspeed"):
            a = forcing.get(n)
            if a is not None:
                a = np.ascontiguousarray(a, np.float64)
                keep.append(a)
                setattr(f, n, _d(a))
        f.forc_row0 = row0
        f.n_rows = next(a.shape[0] for a in keep)
        G = len(self.dom.gauge_node)
        q = np.zeros((n_steps, G))
        tro = np.zeros((n_steps, self.dom.n_cells)) if want_tro else None
        qm = np.zeros((n_steps, self.dom.n_nodes)) if want_qmod else None
        out = getattr(self, "out", None)
        rc = self.L.ora_run_ex(C.byref(self.d), C.byref(self.p), C.byref(self.s), C.byref(f), tt0, n_steps,
                               _d(q), _d(tro), _d(qm), nthreads, C.byref(out) if out is not None else None)
        if rc != 0:
            raise RuntimeError(f"ora_run failed ({rc})")
        return q, tro, qm


# oracle output name -> mhm_eff_params name
MPR_TO_EFF = {"jarvis_c1": "jarvis_thresh_c1", "SMs": "soilMoistSat", "FC": "soilMoistFC", "PW": "wiltingPoint",
              "beta": "soilMoistExp"}


def oracle_mpr(n1: int, H: int, l0, gamma: np.ndarray, offsets, proc_sm: int = 1, proc_pet: int = 0,
               kind: str = "hmath") -> dict:
    """mpr() and its start-up (soil weights, slope_emp) on the CPU for one
    member.  `l0` carries the fields of mhm_l0_desc (mhm_gb300.synth.L0Maps),
    `offsets` the start of each process block in `gamma` (processes 1..10,
    then the total).  Returns the L1 parameters under mhm_eff_params names and
    the start-up products "Wd", "slope_emp", "horizon_depth"."""
    L = load(kind)
    keep = []

    def k(a, dt=np.float64):
        a = np.ascontiguousarray(a, dt)
        keep.append(a)
        return a

    nS, mH = l0.n_soil, l0.max_hor
    hd = k(l0.horizon_depth.copy())
    Wd = k(np.zeros(nS * H * mH))
    rc = L.ora_soil_weights(nS, mH, _i(k(l0.soil_n_hor, np.int32)), _d(k(l0.soil_ud)), _d(k(l0.soil_ld)),
                            _d(k(l0.soil_rz_depth)), H, _d(hd), _d(Wd))
    if rc != 0:
        raise RuntimeError(f"ora_soil_weights failed ({rc})")
    n0 = l0.n_cells0
    se = k(np.zeros(n0))
    L.ora_slope_emp(n0, _d(k(l0.slope0)), _d(se))
    mask = l0.mask0.astype(bool)
    id0 = np.full(mask.size, -1, np.int32)
    id0[mask] = np.arange(n0, dtype=np.int32)
    present = np.zeros(nS, np.int32)
    present[np.unique(l0.soil_id0) - 1] = 1
    g = k(gamma)
    d = OraMprDomain()
    d.nCells0, d.nrows0, d.ncols0, d.nCells1 = n0, l0.nrows0, l0.ncols0, n1
    d.nH, d.nSoil, d.maxHor, d.nGeo = H, nS, mH, l0.n_geo
    d.proc_sm, d.proc_pet = proc_sm, proc_pet
    d.n_soil_params = int(offsets[3] - offsets[2])
    d.fracSealed_cityArea = l0.frac_sealed_city
    d.id0_2d = _i(k(id0, np.int32))
    for n, a in (("up1", l0.l1_up), ("down1", l0.l1_down), ("left1", l0.l1_left), ("right1", l0.l1_right),
                 ("nsub1", l0.l1_nsub), ("LCover0", l0.lcover0), ("soilId0", l0.soil_id0),
                 ("geoUnit0", l0.geo_unit0), ("present", present), ("nHor", l0.soil_n_hor),
                 ("nTill", l0.soil_n_till), ("geoUnitList", l0.geo_unit_list), ("geoUnitKar", l0.geo_unit_kar)):
        setattr(d, n, _i(k(a, np.int32)))
    for n, a in (("Asp0", l0.aspect0), ("y0", l0.y0), ("LAI0", l0.lai0()), ("sand", l0.soil_sand),
                 ("clay", l0.soil_clay), ("DbM", l0.soil_dbm), ("RZdepth", l0.soil_rz_depth)):
        setattr(d, n, _d(k(a)))
    d.slope_emp0 = _d(se)
    d.Wd = _d(Wd)
    d.horizonDepth = _d(hd)
    gm = OraGamma()
    for i, n in enumerate(("interc", "snow", "soil", "runoff", "pet", "interflow", "perc")):
        setattr(gm, n, C.cast(C.byref(g.ctypes.data_as(C.POINTER(C.c_double)).contents, 8 * int(offsets[i])), _dp))
    gm.geo = C.cast(C.byref(g.ctypes.data_as(C.POINTER(C.c_double)).contents, 8 * int(offsets[8])), _dp)
    nl = int(l0.lai0().shape[0])       # LAI entries: 12 monthly slots or a gridded series
    d.nLAI = nl
    sizes = {"maxInter": nl * n1, "petLAIcorFactor": nl * n1, "fRoots": H * n1, "SMs": H * n1, "FC": H * n1,
             "PW": H * n1, "beta": H * n1, "PrieTayAlpha": nl * n1, "aeroResist": nl * n1,
             "surfResist": nl * n1}
    out = {n: np.zeros(sizes.get(n, n1)) for n in MPR_OUT_FIELDS}
    o = OraMprOut(**{n: _d(out[n]) for n in MPR_OUT_FIELDS})
    rc = L.ora_mpr(C.byref(d), C.byref(gm), C.byref(o))
    if rc != 0:
        raise RuntimeError(f"ora_mpr failed ({rc})")
    res = {MPR_TO_EFF.get(n, n): v for n, v in out.items()}
    res["Wd"] = Wd
    res["slope_emp"] = se
    res["horizon_depth"] = hd
    return res
