#!/usr/bin/env python3
"""Benchmark: cell-timesteps/s of the mHM cell chain + mRM routing (FP64).

Default workload (the single large domain): L1 1000 x 1000 cells, 6 soil
horizons, hourly steps, L11 = 4 x 4 L1 cells (62,500 routing nodes, fractal
DEM with a folded main valley: 1478 topological levels).  One benchmark step
advances the whole basin by one chunk of 240 hourly time steps (10 days):
forcing for the chunk (precipitation from a Gaussian random field with a
20-cell length scale, 70 % dry hours, Gamma(0.6, 2 mm/h) amounts; temperature
8 + 10 sin + N(0, 3) degC; Hargreaves PET) is resident in HBM and the cell
chain, the L1->L11 accumulation and the Muskingum routing all run.  Steps
continue the same simulation (states carry over); the forcing window repeats
every step.  Inputs (3 x 1.92 GB of forcing per step) exceed the 129 MB L2,
so no extra L2 flush is needed.  The effective parameters are mpr() of the
parameter namelist's default values over level-0 maps of 2000 x 2000 cells.
The forcing window is generated once on the host from fixed seeds: the GPU
arm, its CPU baseline and the reference arm all run the same arrays.

`value` is device-timed throughput with inputs in HBM; `e2e` is the same run
through the C ABI with the forcing in pinned host memory, copied to the
device inside the timed region (overlapped with compute by the library) and
the gauge discharge copied back every step.

--impl reference times the CPU restatement of the reference (the oracle,
libm build = the C library's exp/log/pow as gfortran calls them, OpenMP over
cells as the reference's own loop, serial routing) on the host cores, whole
240-step chunks of the same workload, each step timed.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-timesteps/s (mHM+mRM, FP64)"
UNIT = "cell-timesteps/s"
CONFIGS = {
    # name: L1 grid, soil horizons, L11 = l11 x l11 L1 cells, L0 = L1 / l0, steps per bench step, DEM
    "large": dict(nrows=1000, ncols=1000, H=6, l11=4, l0=2, chunk=240,
                  dem=dict(dem_kind="fractal", fractal_beta=3.0, tilt=0.0005, ridges=6)),
    "medium": dict(nrows=500, ncols=500, H=6, l11=4, l0=2, chunk=240,
                   dem=dict(dem_kind="fractal", fractal_beta=3.0, tilt=0.0005, ridges=3)),
    "small": dict(nrows=96, ncols=96, H=3, l11=4, l0=4, chunk=240, dem=dict(dem_kind="plane")),
}
ALG_BYTES_PER_CELL_STEP = 32  # 24 B forcing read + 8 B total runoff write
# generator seeds of every synthetic input (numpy.random.default_rng)
SEEDS = {"domain_dem": 1, "forcing": 2, "ensemble_parameter_sets": 3, "l0_maps": 4}
LAND_COVER_MAPPING = ("5 synthetic L0 land-cover classes -> mHM land-cover codes "
                      "{1: 1 forest, 2: 1 forest, 3: 3 pervious, 4: 3 pervious, 5: 2 impervious}")


def _env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def replica_throughput(local_ms: float, units_per_rank: float, world: int, device=None) -> tuple[float, float]:
    """(job ms, whole-job units/s) of `world` independent replicas: the
    slowest rank's time (all-reduce MAX over the process group when
    world > 1) against the units of all ranks."""
    ms = float(local_ms)
    if world > 1:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, units_per_rank * world / (ms * 1e-3)


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[4:8]):
                if v.strip().lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except json.JSONDecodeError:
            pass
    return {}


def run_manifest(device, lib) -> dict:
    """What the numbers were measured on: the GPU, its driver, the CUDA and
    PyTorch runtimes, the library variant loaded and the host."""
    import platform
    import subprocess

    import torch
    props = torch.cuda.get_device_properties(device)
    driver = None
    try:
        r = subprocess.run(["nvidia-smi", "-i", str(device.index or 0), "--query-gpu=driver_version",
                            "--format=csv,noheader"], capture_output=True, text=True, timeout=20)
        driver = r.stdout.strip() or None
    except (OSError, subprocess.SubprocessError):
        pass
    from mhm_gb300 import _lib
    return {"gpu": props.name, "sm_count": props.multi_processor_count, "compute_capability": f"{props.major}.{props.minor}",
            "hbm_gib": round(props.total_memory / 2**30, 1), "driver": driver, "cuda_runtime": torch.version.cuda,
            "torch": torch.__version__, "library": _lib.lib_path().name,
            "bounds_checked": bool(lib.mhm_bounds_checked()), "host": platform.machine(),
            "python": platform.python_version()}


def profile_figure(key: str, name: str = "cell_chain_kernel_H6_hourly.md"):
    """A per-cell-step figure ("<key>: <value>") of the cell-chain kernel from
    the committed ncu summary."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def traffic_from_profiles(name: str):
    """DRAM bytes per cell-step of the cell-chain kernel from the committed ncu summary."""
    return profile_figure("dram_bytes_per_cell_step", name)


def build_workload(cfg_name: str, order=None):
    """(domain, L0 maps, parameter vector, steps per bench step): the basin
    of the configuration, its level-0 maps under L1 = L0 x l0 and the
    parameter namelist's default values (mhm_parameter.nml `value` column),
    which mpr() turns into the effective parameters.  `order` computes the
    routing order (the CPU arms pass the oracle's)."""
    from mhm_gb300 import params, synth
    c = CONFIGS[cfg_name]
    dom = synth.make_domain(c["nrows"], c["ncols"], c["H"], c["l11"], seed=SEEDS["domain_dem"], order=order,
                            **c["dem"])
    l0 = synth.make_l0(dom, c["l0"], seed=SEEDS["l0_maps"])
    gamma = params.default_gamma(1, 0, 1, l0.n_geo)
    return dom, l0, gamma, c["chunk"]


def workload_config(cfg_name: str, dom, chunk: int) -> dict:
    """The `config` object of both arms (the same dict for the same workload)."""
    c = CONFIGS[cfg_name]
    levels = dom.depth_stats()[0]
    return {"workload": f"single large domain: L1 {dom.nrows}x{dom.ncols} ({dom.n_cells} cells), "
                        f"{dom.n_horizons} soil horizons, hourly, L11 {dom.n_nodes} nodes ({levels} routing "
                        f"levels); step = {chunk} time steps" if cfg_name == "large" else
                        f"{cfg_name}: L1 {dom.nrows}x{dom.ncols}, {dom.n_horizons} horizons; step = {chunk} steps",
            "cells": dom.n_cells, "horizons": dom.n_horizons, "l11_nodes": dom.n_nodes, "routing_levels": levels,
            "l0_cells": dom.n_cells * c["l0"] ** 2, "steps_per_bench_step": chunk,
            "parameters": "mpr() of the parameter namelist's default values (processes 1,1,1,1,0,1,1,1,1,0)",
            "forcing": f"one {chunk}-step hourly window, repeated every step (states carry over): precipitation "
                       "occurrence from a Gaussian random field (20-cell length scale, 70 % dry hours), "
                       "Gamma(0.6, 2 mm/h) amounts; temperature 8 + 10 sin + N(0, 3) degC; Hargreaves PET",
            "seeds": SEEDS, "land_cover_mapping": LAND_COVER_MAPPING,
            "parallelism": "single GPU",
            "l2": ("inputs larger than L2 (forcing 3 x %.2f GB per step)" if 3 * chunk * dom.n_cells * 8 > 129e6
                   else "inputs smaller than L2 (forcing 3 x %.2f GB per step)") % (chunk * dom.n_cells * 8 / 1e9)}


def host_forcing(dom, chunk: int, pinned: bool):
    """The forcing window every arm uses (same seed -> same arrays): numpy
    views, in pinned host memory when `pinned`."""
    from mhm_gb300 import synth
    if pinned:
        import torch
        bufs = {k: torch.empty((chunk, dom.n_cells), dtype=torch.float64, pin_memory=True)
                for k in ("pre", "temp", "pet")}
        out = {k: v.numpy() for k, v in bufs.items()}
    else:
        bufs, out = None, None
    f = synth.make_forcing_grf(dom, chunk, seed=SEEDS["forcing"], out=out)
    return f, bufs


def run_gpu(args) -> dict:
    import torch
    from mhm_gb300._lib import load
    from mhm_gb300.model import MhmGpu

    rank, world, local = _env_rank()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(device)
    lib = load()
    dom, l0, gamma, chunk = build_workload(args.config)
    N = dom.n_cells
    g = MhmGpu(dom, proc_soilmoist=1, proc_pet=0, device=device.index)
    g.mpr_setup(l0)
    g.mpr(gamma)                      # effective parameters and Muskingum coefficients
    g.init_states(0)
    hf, pinned = host_forcing(dom, chunk, pinned=True)
    pre, temp, pet = (pinned[k].to(device) for k in ("pre", "temp", "pet"))
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(g.stream, device=device)
    g.set_meteo(1, pre, temp, pet, on_device=True)
    tune = None if args.no_autotune else g.autotune(1, chunk)   # register variant x routing sub-chunk

    G = len(dom.gauge_node)
    qbufs = [np.zeros((1, G, chunk)) for _ in range(2)]

    def step(s: int, on_device=True):
        """Enqueue one benchmark step (the library pipelines consecutive steps:
        routing of step s overlaps the cell chain of step s+1); the gauge
        series lands in a host buffer when g.sync() returns."""
        tt0 = 1 + s * chunk
        if on_device:
            g.set_meteo(tt0, pre, temp, pet, on_device=True)
        else:
            g.set_meteo(tt0, hf["pre"], hf["temp"], hf["pet"])
        g.run_async(tt0, chunk, qbufs[s & 1])

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # FP64 issue-rate peak on this GPU (roofline denominator for the FP64 pipe)
    import ctypes as C
    fl = C.c_double()
    fp64_peak = None
    if lib.mhm_probe_fp64(20000, C.byref(fl)) == 0:
        fp64_peak = fl.value
    for s in range(args.warmup):
        step(s)
    g.sync()
    torch.cuda.synchronize()
    g.set_timing(True)
    launches0 = lib.mhm_kernel_launch_count()
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(device.index) as clk:
        ev0.record(stream)
        for s in range(args.warmup, args.warmup + args.steps):
            step(s)
        g.sync()  # joins the routing stream into the library stream
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = lib.mhm_kernel_launch_count() - launches0
    n_cell, t_cell = g.get_timing(0)
    n_acc, t_acc = g.get_timing(1)
    n_rt, t_rt = g.get_timing(2)
    g.set_timing(False)
    ms, value = replica_throughput(ms, float(N) * chunk * args.steps, world, device)

    # ---- e2e: host forcing (pinned), H2D + compute + D2H of the gauge series per step ----
    e2e_steps = 16  # whole steps, so that filling and draining the copy / routing pipeline is amortised
    step(args.warmup + args.steps, on_device=False)  # warm the staging buffers
    g.sync()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(e2e_steps):
        step(args.warmup + args.steps + 1 + s, on_device=False)
    g.sync()  # all H2D copies, compute and gauge D2H copies complete
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    wall_ms = (time.perf_counter() - t0) * 1e3
    e2e_ms = max(e2e_ms, wall_ms)  # host copies happen inside mhm_run; count whichever is longer
    e2e_ms, e2e_value = replica_throughput(e2e_ms, float(N) * chunk * e2e_steps, world, device)

    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    per_launch_s = (t_cell / max(n_cell, 1)) * 1e-3
    alg_bytes = ALG_BYTES_PER_CELL_STEP * N * chunk
    achieved = alg_bytes / per_launch_s / 1e9
    tb = traffic_from_profiles("cell_chain_kernel_H6_hourly.md")
    fp64_line = {"peak": fp64_peak / 1e12 if fp64_peak else None, "unit": "TFLOP/s",
                 "peak_source": "measured live (DFMA probe, 2 FLOP per DFMA)"}
    ops = traffic_from_profiles_ops()
    pipe_ops = profile_figure("fp64_pipe_ops_per_cell_step")
    if fp64_peak and ops:
        flops = ops * N * chunk / per_launch_s
        fp64_line.update({"achieved": flops / 1e12, "frac": flops / fp64_peak, "flop_per_cell_step": ops,
                          "kernel": "cell_chain_kernel<6>"})
    if fp64_peak and pipe_ops:
        # occupancy of the FP64 pipe: a DADD or DMUL takes a full slot, as a
        # DFMA does, so the operations count against the DFMA issue rate
        fp64_line.update({"pipe_ops_per_cell_step": pipe_ops,
                          "pipe_frac": pipe_ops * N * chunk / per_launch_s / (fp64_peak / 2.0)})
    # the roof that binds the kernel: warp instructions issued (4 schedulers per SM,
    # one instruction each per cycle) at the SM clock sampled under load
    wi = profile_figure("warp_inst_per_cell_step")
    n_sm = torch.cuda.get_device_properties(device).multi_processor_count
    sm_mhz = clk.summary().get("sm_mhz") or None
    issue_line = None
    if wi and sm_mhz:
        ach = wi * N * chunk / per_launch_s
        peak = 4.0 * n_sm * sm_mhz * 1e6
        issue_line = {"achieved": ach, "peak": peak, "unit": "warp-inst/s", "frac": ach / peak,
                      "warp_inst_per_cell_step": wi, "kernel": "cell_chain_kernel<6>",
                      "peak_source": f"{n_sm} SMs x 4 issue slots x sampled SM clock {sm_mhz:.0f} MHz"}
    cfg = workload_config(args.config, dom, chunk)
    if world > 1:
        cfg["parallelism"] = f"replicas x{world}"
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 3 * chunk * N * 8,
                "d2h_bytes_per_step": chunk * len(dom.gauge_node) * 8, "steps": e2e_steps},
        "gpu_launches": int(launches),
        # the contract's HBM view of the dominant kernel; the roofs that bind
        # it are the FP64 pipe and the instruction issue rate
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": (tb * N * chunk) if tb else None,
                     "kernel": "cell_chain_kernel<6>", "alg_bytes_per_launch": alg_bytes,
                     "launch_ms": per_launch_s * 1e3, "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)"
                     if peaks else "of fallback",
                     "binding_roof": "the FP64 pipe (roofline_fp64.pipe_frac) and instruction issue "
                                     "(roofline_issue); HBM is not the limit"},
        "roofline_fp64": fp64_line,
        "roofline_issue": issue_line,
        "kernel_time_ms": {"cell_chain": t_cell, "runoff_acc": t_acc, "routing": t_rt,
                           "timed_region": ms},
        "clocks": clk.summary(),
        "autotune": tune,
        "manifest": run_manifest(device, lib),
    }
    g.close()
    del pre, temp, pet
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_ensemble:
        out["batched"] = run_ensemble(args, device)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(dom, l0, gamma, hf, chunk, args)
    if rank == 0 and not args.no_serving:
        out["serving"] = run_serving(args)
    if rank == 0 and not args.no_uneven:
        t0 = time.perf_counter()
        out["uneven"] = run_uneven(args, side_by_side=False)   # fused rounds vs one basin at a time
        out["uneven"]["wall_s"] = time.perf_counter() - t0
    if world > 1:
        torch.distributed.destroy_process_group()
    return out if rank == 0 else None


ENSEMBLE = dict(nrows=200, ncols=200, H=3, l11_factor=4, l0_factor=4, members=256, chunk=240)


def run_ensemble(args, device, plain_members: int = 8) -> dict:
    """The calibration-ensemble workload: L1 200 x 200 (40,000 cells), 3 soil
    horizons, L0 = L1/4, 256 parameter sets drawn uniformly within the
    namelist bounds, hourly.  Batched: one context holds all 256 members
    (device MPR for all of them in one call, one cell-chain launch per chunk
    over member x cell, routing of all members per wavefront tick).  Plain:
    the one-parameter-set drop-in, members one after another (each with its
    own MPR and run), timed on `plain_members` members.  Both advance every
    member by the same chunks of 240 steps; throughput counts member x cell x
    step."""
    import torch
    from mhm_gb300 import params as gparams
    from mhm_gb300 import synth
    from mhm_gb300.model import MhmGpu
    E = ENSEMBLE
    dom = synth.make_domain(E["nrows"], E["ncols"], E["H"], E["l11_factor"], seed=1, dem_kind="fractal",
                            fractal_beta=3.0, tilt=0.001)
    l0 = synth.make_l0(dom, E["l0_factor"], seed=4)
    M, chunk, N = (args.ensemble_members or E["members"]), E["chunk"], dom.n_cells
    gam = gparams.random_gammas(M, 1, 0, 1, l0.n_geo, seed=3)
    fh = synth.make_forcing(dom, chunk, seed=SEEDS["forcing"])   # i.i.d. hourly forcing of the plain basin
    pre, temp, pet = (torch.from_numpy(fh[k]).to(device) for k in ("pre", "temp", "pet"))
    G = len(dom.gauge_node)
    K = max(1, min(args.steps, 3))

    def timed(g, q, n_steps, first_step):
        stream = torch.cuda.ExternalStream(g.stream, device=device)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in range(first_step, first_step + n_steps):
            g.set_meteo(1 + s * chunk, pre, temp, pet, on_device=True)
            g.run_async(1 + s * chunk, chunk, q[s & 1])
        g.sync()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    # batched
    g = MhmGpu(dom, proc_soilmoist=1, proc_pet=0, n_members=M, device=device.index)
    g.mpr_setup(l0)
    g.mpr(gam)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.mpr(gam)
    mpr_ms = (time.perf_counter() - t0) * 1e3
    for m in range(M):
        g.init_states(m)
    g.set_meteo(1, pre, temp, pet, on_device=True)
    tune = None if args.no_autotune else g.autotune(1, 48)
    qb = [np.zeros((M, G, chunk)) for _ in range(2)]
    timed(g, qb, 2, 0)                      # warm-up
    ms_b = timed(g, qb, K, 2)
    g.close()
    vb = float(M) * N * chunk * K / (ms_b * 1e-3)
    if args.ensemble_no_plain:
        return {"workload": f"calibration ensemble: L1 {E['nrows']}x{E['ncols']} ({N} cells), {M} parameter sets",
                "value": vb, "unit": UNIT, "members": M, "ms_batched": ms_b, "autotune_batched": tune}
    # plain: one member per run, one after another
    p = MhmGpu(dom, proc_soilmoist=1, proc_pet=0, n_members=1, device=device.index)
    p.mpr_setup(l0)
    qp = [np.zeros((1, G, chunk)) for _ in range(2)]
    p.mpr(gam[0])
    p.init_states(0)
    p.set_meteo(1, pre, temp, pet, on_device=True)
    tune_p = None if args.no_autotune else p.autotune(1, 48)
    timed(p, qp, 2, 0)                      # warm-up
    ms_p, mpr_p = 0.0, 0.0
    for m in range(plain_members):
        t0 = time.perf_counter()
        p.mpr(gam[m])
        mpr_p += (time.perf_counter() - t0) * 1e3
        p.init_states(0)
        ms_p += timed(p, qp, K, 0)
    p.close()
    vp = float(plain_members) * N * chunk * K / (ms_p * 1e-3)
    return {"workload": f"calibration ensemble: L1 {E['nrows']}x{E['ncols']} ({N} cells), {E['H']} soil horizons, "
                        f"L0 = L1/{E['l0_factor']}, {M} parameter sets within the namelist bounds, hourly, "
                        f"{dom.n_nodes} L11 nodes; {K} chunks of {chunk} steps per member",
            "value": vb, "unit": UNIT, "plain_value": vp, "speedup_vs_plain": vb / vp, "members": M,
            "plain_members_timed": plain_members, "ms_batched": ms_b, "ms_plain": ms_p,
            "mpr_ms_all_members": mpr_ms, "mpr_ms_per_member_plain": mpr_p / plain_members,
            "autotune_batched": tune, "autotune_plain": tune_p}


def run_serving(args) -> dict:
    """The serving workload: a catalogue of basins (cell counts log-uniform in
    1e3..1e6, 2-6 soil horizons, each with its own D8 network), Poisson
    arrivals at each rate, each request a random parameter vector within the
    namelist bounds, a 30..365-day hourly horizon and a warm start from the
    basin's device-resident 90-day spin-up; HBM budget 150 GB.  The server
    (continuous batching) and the one-run-at-a-time path serve the same
    request stream; p50/p99 latency and cell-step throughput for both."""
    import torch
    from mhm_gb300 import serve
    torch.cuda.set_device(0)
    t_start = time.perf_counter()
    basins = serve.make_catalogue(args.serve_basins, seed=11, include_max=True)   # up to 1e6 cells
    cells = [b.n_cells for b in basins]
    out = {"metric": "serving: p50/p99 latency [s] and cell-timesteps/s (mHM+mRM, FP64)", "unit": "s",
           "catalogue": [b.name for b in basins], "cells_min": int(min(cells)), "cells_max": int(max(cells)),
           "hbm_budget_gb": 150, "requests_per_rate": args.serve_requests,
           "horizon_days": [30, 365], "rates": []}
    srv = serve.Server(basins, hbm_budget=150e9, chunk=240, max_slots=16)   # spin-ups, forcing windows
    srv.close()
    for rate in args.serve_rates:
        reqs = serve.make_requests(basins, args.serve_requests, rate, seed=int(rate))
        srv = serve.Server(basins, hbm_budget=150e9, chunk=240, max_slots=16, fused=True)
        batched = srv.serve(reqs, timeout_s=1800)
        srv.close()
        plain_reqs = serve.make_requests(basins, args.serve_requests, rate, seed=int(rate))
        plain = serve.serve_plain(basins, plain_reqs, 240)
        same = all(np.array_equal(a.discharge(), b.discharge()) for a, b in zip(
            sorted(reqs, key=lambda r: r.rid), sorted(plain_reqs, key=lambda r: r.rid)))
        out["rates"].append({"rate_per_s": rate, "batched": batched, "plain": plain,
                             "throughput_ratio": batched["throughput"] / plain["throughput"],
                             "results_identical": bool(same)})
    out["wall_s"] = time.perf_counter() - t_start
    return out


def run_uneven(args, side_by_side: bool = True) -> dict:
    """Batched uneven basins: 64 basins with cell counts log-uniform in
    1e3..2.5e5, 2-6 soil horizons, 90..730-day hourly horizons, each with its
    own D8 network, all submitted at once.  Fused (the headline): rounds of
    one chunk, each ONE persistent cell-chain launch over every basin still
    running (a device work queue of tiles), routing per basin on its own
    streams (serve.run_batched).  Side by side: the serving loop, one launch
    per basin context (autotuned per basin).  Plain: the basins one after
    another."""
    import torch
    from mhm_gb300 import serve
    torch.cuda.set_device(0)
    basins = serve.make_catalogue(args.uneven_basins, seed=21, n_min=1e3, n_max=2.5e5)
    rng = np.random.default_rng(22)
    from mhm_gb300 import params as gparams
    reqs, reqs_p = [], []
    for i, b in enumerate(basins):
        g = gparams.random_gammas(1, 1, 0, 1, b.l0.n_geo, seed=300 + i)[0]
        days = int(rng.integers(90, 731))
        reqs.append(serve.Request(rid=i, basin=i, gamma=g, horizon=24 * days))
        reqs_p.append(serve.Request(rid=i, basin=i, gamma=g, horizon=24 * days))
    def fresh():
        return [serve.Request(rid=r.rid, basin=r.basin, gamma=r.gamma, horizon=r.horizon) for r in reqs]

    # fused: rounds of one persistent cell-chain launch over every basin
    # still running (a device work queue of tiles), routing per basin
    srv = serve.Server(basins, hbm_budget=150e9, chunk=240, max_slots=1, spinup_steps=0)   # spin-up / windows
    srv.close()
    fused = serve.run_batched(basins, reqs, 240)
    # side by side: the serving loop, one launch per basin context on its own streams
    streams, tuned, reqs_s = None, None, None
    if side_by_side:
        reqs_s = fresh()
        srv = serve.Server(basins, hbm_budget=150e9, chunk=240, max_slots=1, spinup_steps=0, autotune=True)
        streams = srv.serve(reqs_s, timeout_s=3000)
        tuned = srv.tuned
        srv.close()
    plain = serve.serve_plain(basins, reqs_p, 240)
    same = all(np.array_equal(a.discharge(), b.discharge()) and (c is None or np.array_equal(a.discharge(),
                                                                                          c.discharge()))
               for a, b, c in zip(reqs, reqs_p, reqs_s or [None] * len(reqs)))
    cells = [b.n_cells for b in basins]
    return {"metric": "batched uneven basins: cell-timesteps/s (mHM+mRM, FP64)", "unit": UNIT,
            "basins": len(basins), "cells_min": int(min(cells)), "cells_max": int(max(cells)),
            "horizons": [b.dom.n_horizons for b in basins],
            "routing_levels": [b.dom.depth_stats()[0] for b in basins],
            "value": fused["throughput"], "plain_value": plain["throughput"],
            "speedup_vs_plain": fused["throughput"] / plain["throughput"],
            "side_by_side_value": streams["throughput"] if streams else None,
            "makespan_s": fused["wall_s"], "side_by_side_makespan_s": streams["wall_s"] if streams else None,
            "plain_makespan_s": plain["wall_s"], "results_identical": bool(same), "autotune_side_by_side": tuned}


def traffic_from_profiles_ops():
    return profile_figure("fp64_flop_per_cell_step")


class OracleArm:
    """The CPU restatement of the reference's path on this host: the oracle
    (libm build: the C library's exp/log/pow as gfortran calls them) runs
    mpr() of the same parameter vector and then the time loop -- OpenMP over
    cells as the reference's own `!$OMP do schedule(static)` over L1 cells,
    serial routing -- on the same forcing window as the GPU arm."""

    def __init__(self, dom, l0, gamma, forcing):
        from mhm_gb300 import params
        from oracle import oracle
        off = params.offsets(1, 0, 1, l0.n_geo)
        t0 = time.perf_counter()
        eff = oracle.oracle_mpr(dom.n_cells, dom.n_horizons, l0, gamma, off, 1, 0, "libm")
        self.mpr_s = time.perf_counter() - t0
        eff = {k: v for k, v in eff.items() if k not in ("Wd", "slope_emp", "horizon_depth")}
        self.run = oracle.OracleRun(dom, eff, rout_param=gamma[off[7]:off[7] + 5], kind="libm")
        self.f = forcing
        self.dom = dom
        self.tt = 1

    def chunk(self, n_steps: int, threads: int) -> float:
        """Advance n_steps (the forcing window's first n_steps rows, as the GPU
        arm repeats its window); returns the wall seconds."""
        f = {k: v[:n_steps] for k, v in self.f.items()}
        t0 = time.perf_counter()
        self.run.run(f, self.tt, self.tt, n_steps, nthreads=threads)
        dt = time.perf_counter() - t0
        self.tt += n_steps
        return dt


def cpu_baseline(dom, l0, gamma, forcing, chunk: int, args, target_s: float = 12.0) -> dict:
    """The oracle on a bounded sample of the bench workload (same basin,
    parameters and forcing window): one untimed chunk (SM initialisation),
    then whole chunks on all host threads until ~target_s, and a 24-step
    sample on one thread."""
    threads = os.cpu_count() or 1
    arm = OracleArm(dom, l0, gamma, forcing)
    arm.chunk(chunk, threads)
    done, spent = 0, 0.0
    while spent < target_s or done == 0:
        spent += arm.chunk(chunk, threads)
        done += chunk
    one = arm.chunk(24, 1)
    return {"value": dom.n_cells * done / spent, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{dom.n_cells} cells x {done} hourly steps ({done // chunk} whole {chunk}-step chunks of "
                      f"the bench workload, same forcing window and parameters) in {spent:.1f} s; oracle libm "
                      f"build, OpenMP {threads} threads over cells, serial routing",
            "one_thread": {"value": dom.n_cells * 24 / one, "unit": UNIT, "cores": 1,
                           "sample": f"{dom.n_cells} cells x 24 hourly steps in {one:.1f} s"},
            "mpr_s": arm.mpr_s}


def run_reference(args) -> dict | None:
    """--impl reference: the reference's CPU path (the oracle port: no
    Fortran compiler exists here or on the GPU host, so the reference
    itself cannot be built) on this host's cores, on the GPU arm's workload:
    the same basin (routing order from the oracle's restatement of
    L11_routing_order), mpr() of the same default parameters, the same
    forcing window.  Every step advances the whole basin by one chunk on all
    host threads, exactly as one GPU step does; W untimed steps, then K timed
    ones, each timed on its own."""
    rank, world, _ = _env_rank()
    if rank != 0:
        return None
    from oracle import oracle
    oracle.build()
    dom, l0, gamma, chunk = build_workload(args.config, order=lambda f, t, n, o: oracle.routing_order(f, t, n, o))
    forcing, _ = host_forcing(dom, chunk, pinned=False)
    threads = os.cpu_count() or 1
    arm = OracleArm(dom, l0, gamma, forcing)
    for _ in range(args.warmup):
        arm.chunk(chunk, threads)
    per = [arm.chunk(chunk, threads) for _ in range(args.steps)]
    one = arm.chunk(24, 1)
    total = sum(per)
    v = dom.n_cells * chunk * args.steps / total
    base = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{args.steps} whole {chunk}-step chunks of {dom.n_cells} cells, each timed "
                      f"(min {min(per):.2f} s, max {max(per):.2f} s); oracle libm build, OpenMP {threads} threads "
                      f"over cells, serial routing",
            "one_thread": {"value": dom.n_cells * 24 / one, "unit": UNIT, "cores": 1,
                           "sample": f"{dom.n_cells} cells x 24 hourly steps in {one:.1f} s"}}
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.config, dom, chunk),
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="large", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--ensemble-only", action="store_true", help="only the batched-ensemble measurement")
    ap.add_argument("--ensemble-members", type=int, default=0, help="members of the ensemble (default 256)")
    ap.add_argument("--ensemble-no-plain", action="store_true", help="skip the one-set-at-a-time comparison")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the kernel variant of MHM_CELL_OCC / MHM_ROUTE_SUB (for profiling)")
    ap.add_argument("--serve", action="store_true", help="measure the serving loop instead (p50/p99 latency)")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[50.0, 100.0])
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-basins", type=int, default=12)
    ap.add_argument("--no-serving", action="store_true", help="skip the serving measurement of the default run")
    ap.add_argument("--uneven", action="store_true", help="measure the batched uneven-basins workload instead")
    ap.add_argument("--uneven-basins", type=int, default=64)
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-basins measurement of the default run")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.serve:
        print(json.dumps(run_serving(args)))
        return
    if args.uneven:
        print(json.dumps(run_uneven(args)))
        return
    if args.ensemble_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(run_ensemble(args, torch.device("cuda", 0))))
        return
    out = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
