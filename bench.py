"""Benchmark of the GB300 GOLDSTEIN tracer step (one JSON line on rank 0).

Workloads (seeded synthetic members with the reference's grid formulas):
  c3  (default) batched ensemble: 256 members split evenly among 18x18x16,
      36x36x16 and 36x36x32 grids, 2-24 tracers each, per-member diffusivities,
      masks and velocities; FP32 transfers, FP64 state; every step one CUDA
      graph replay (the transfer kernels, the exact convective adjustment and
      the scale update)
  c2  single member 36x36x16, 17 tracers, isoneutral branch on, FP64 plain form
  c1  single member 36x36x16, 2 tracers, FP64 plain form
  c5  single grid 360x180x32, 24 tracers (HBM stress test), FP64 plain form or, with
      --precision fp32flux, the split-precision form
  bg5 the BIOGEM tracer coupling (biogem_tracercoupling) on the c5 grid with 8 particulate
      tracers: a step is one coupling of the device-resident GOLDSTEIN and BIOGEM fields;
      `value` is tracer cell-couplings/s (one tracer of one wet cell coupled)
  ea64 the EMBM atmosphere step (tstipa) on a 64x64 surface grid, one launch per step as
      the model calls it; `value` is air cell-updates/s
  ea36e the EMBM step of a 256-member ensemble of 36x36 surface grids, one launch per step
      for all members (gb_ea_step_many)
  ice64 step_seaice on a 64x64 grid: the implicit sea-ice transport (tstipsic) with its
      diagnostics, then the post-processing (area clamp, thin-ice removal and its fluxes), two
      launches per step; `value` is ice cell-updates/s (two tracers per cell)
  ocean36 the device-resident ocean step of a 36x36x16 basin with 8 tracers: momentum, then
      tstepo (split-precision form), and the BIOGEM tracer coupling every 5th step; `value` is
      tracer cell-updates/s of the whole step
  ocean5 the same ocean step at the stress-test size, 360x180x32 with 24 tracers and the
      stress test's stable time step (1/2400 yr; 65,160 streamfunction points: the
      block-tridiagonal streamfunction solve)
  mo36 the momentum step (wind, jbar, streamfunction, islands, velc) of a 36x36x16 basin
      with two islands, on the density of an FP64 handle; `value` is wet-cell momentum
      updates/s (each wet cell's u, v, w advanced one step)
      (two tracers of one surface cell advanced one step)

A step is one tracer timestep (tstepo) of every member.  `value` is tracer
cell-updates/s with the state resident in HBM (c3: the 256 states, 2 x 0.6 GB,
are larger than L2, so L2 is not flushed; c1/c2: L2 flushed before every step).
For c3 the line also gives the plain per-member GPU rate (the FP64 drop-in path
stepping the members one at a time) and the largest per-tracer error of the
batched result against that FP64 path (bit-identical to the FP64 oracle) on a
sample of members.  `e2e` is the whole job through the C-ABI with host buffers:
c3 admits the 256 members from host arrays (gb_ens_add), steps them and downloads
every member (gb_ens_download); c1/c2 upload the forcing and velocities and read
rho back every step.

--impl reference times the reference algorithm on the host cores instead (the
oracle's C restatement of goldstein.f90:2280-2842 with the reference's dead
copies, one member per process, all host cores).  Multi-GPU (torchrun): every
rank runs an independent replica (members are independent), weak scaling, time
= max over ranks.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "c1": dict(name="tstepo_fp64_36x36x16_L2", factory="config_c1"),
    "c2": dict(name="tstipo_diso_fp64_36x36x16_L17", factory="config_c2"),
    "c3": dict(name="ensemble256_fp32flux_18x18x16_36x36x16_36x36x32_L2-24", members=256, seed=3),
    "c5": dict(name="stress_360x180x32_L24", factory="config_c5"),
    "bg5": dict(name="biogem_tracercoupling_360x180x32_L24_sed8", factory="config_c5", n_l_sed=8),
    "ea64": dict(name="embm_tstipa_64x64", maxi=64, maxj=64),
    "ea36e": dict(name="embm_tstipa_ensemble256_36x36", maxi=36, maxj=36, members=256),
    "ice64": dict(name="seaice_step_seaice_64x64", maxi=64, maxj=64, kind="ice"),
    "mo36": dict(name="momentum_36x36x16_2islands", maxi=36, maxj=36, maxk=16),
    "rs5": dict(name="goldstein_restart_write_360x180x32_L24", factory="config_c5"),
    "rs5s": dict(name="goldstein_restart_write_360x180x32_L2", factory="config_c5", maxl=2),
    "ocean36": dict(name="ocean_step_36x36x16_L8_momentum_tracers_biogem", maxi=36, maxj=36, maxk=16, maxl=8,
                    couple_every=5),
    "ocean5": dict(name="ocean_step_360x180x32_L24_momentum_tracers_biogem", maxi=360, maxj=180, maxk=32, maxl=24,
                   couple_every=5, cpu_steps=3, member_kw=dict(nyear=2400, diff_h=1000.0)),
}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d.get(workload, {}).get(kernel)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 50 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(m) -> int:
    """Bytes one step must move at minimum: FP64 state read once and written once,
    u(3) read once per wet cell, k1 once (16*L*N_wet + 24*N_wet + 4*(maxi+2)*(maxj+2))."""
    nw = m.wet_cells
    return 16 * m.maxl * nw + 24 * nw + 4 * (m.maxi + 2) * (m.maxj + 2)


def cpu_baseline(m, target_s: float = 12.0):
    """Time the oracle (serial, 1 core) on a bounded number of steps of the same member."""
    from oracle import oracle_lib
    s = oracle_lib.OracleState(m)
    s.step(1)
    t0 = time.perf_counter()
    s.step(2)
    per = (time.perf_counter() - t0) / 2
    n = max(3, min(2000, int(target_s / max(per, 1e-6))))
    s = oracle_lib.OracleState(m)
    t0 = time.perf_counter()
    s.step(n, faithful=True)
    dt = time.perf_counter() - t0
    cu = m.wet_cells * m.maxl * n
    return {"value": cu / dt, "unit": "tracer cell-updates/s", "cores": 1, "kind": "port",
            "sample": f"{n} steps of the same member, oracle C restatement with the reference's dead copies, -O2"}


def _ensemble_members(n: int, seed: int):
    from cgenie_gb300 import grid
    return [grid.make_member(c) for c in grid.ensemble_configs(n, seed=seed)]


def _oracle_worker(job):
    """Step a share of the ensemble members with the oracle (one process); returns
    (tracer cell-updates, seconds) of the timed steps."""
    idx, n, seed, warmup, steps, faithful = job
    sys.path.insert(0, ROOT)
    from cgenie_gb300 import grid
    from oracle import oracle_lib
    cfgs = grid.ensemble_configs(n, seed=seed)
    states = [oracle_lib.OracleState(grid.make_member(cfgs[i])) for i in idx]
    for st in states:
        st.step(warmup, faithful=faithful)
    cu = sum(st.m.wet_cells * st.m.maxl for st in states) * steps
    t0 = time.perf_counter()
    for st in states:
        st.step(steps, faithful=faithful)
    return cu, time.perf_counter() - t0


def oracle_pool_rate(n: int, seed: int, warmup: int, steps: int, faithful: bool = True):
    """Ensemble throughput of the oracle on every host core (one process per core, the
    members dealt round-robin); the slowest process sets the time."""
    import multiprocessing as mp
    procs = max(1, os.cpu_count() or 1)
    jobs = [(list(range(p, n, procs)), n, seed, warmup, steps, faithful) for p in range(procs)]
    jobs = [j for j in jobs if j[0]]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        res = pool.map(_oracle_worker, jobs)
    cu = sum(r[0] for r in res)
    dt = max(r[1] for r in res)
    return cu / dt, len(jobs), cu // max(1, steps)


def bg_algorithmic_bytes(wet_cells: int, L: int, Ls: int) -> int:
    """Bytes one coupling must move: per wet cell read go_ts, vocn, vdocn (3L), mass, volume,
    rmass (3), vbio_part, vdbio_part (2Ls); write vocn, ts, ts1 (3L), mass, rmass (2),
    vbio_part (Ls) -- 8 * (6L + 3Ls + 5) bytes."""
    return 8 * (6 * L + 3 * Ls + 5) * wet_cells


def bg_cpu_rate(m, st, target_s: float = 12.0):
    """The oracle's coupling (serial, 1 core) on the same fields: (cell-couplings/s, calls)."""
    from oracle import oracle_lib
    go = oracle_lib.go_ts_interior(m.ts)
    a = st.copy()
    t0 = time.perf_counter()
    oracle_lib.bg_tracercoupling(m, a, go)
    per = time.perf_counter() - t0
    n = max(1, min(50, int(target_s / max(per, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(n):
        go, _ = oracle_lib.bg_tracercoupling(m, a, go)   # successive couplings of the evolving fields
    dt = time.perf_counter() - t0
    return m.wet_cells * m.maxl * n / dt, n


def run_bg(args, rank, world, local, dist):
    """The BIOGEM tracer coupling on the c5 grid: device-resident timing, end to end, roofline."""
    import ctypes as C

    import numpy as np
    import torch
    from cgenie_gb300 import biogem, grid
    from cgenie_gb300.goldstein import kernel_launch_count, new_member_run
    w = WORKLOADS[args.workload]
    m = grid.make_member(getattr(grid, w["factory"])())
    Ls = w["n_l_sed"]
    st = biogem.make_state(m, n_l_sed=Ls, seed=5)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g = new_member_run(m, device=local, stream=stream.cuda_stream)
    g.tstepo(1)
    bg = biogem.BiogemCoupling(m, n_l_sed=Ls, device=local)
    bg.upload(st)
    bg.set_increments(st)
    for _ in range(args.warmup):
        bg.tracercoupling(g)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = kernel_launch_count()
    for s in range(args.steps):
        starts[s].record(stream)
        bg.tracercoupling(g)
        ends[s].record(stream)
    torch.cuda.synchronize()
    launches = kernel_launch_count() - n0
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    total_ms = float(sum(a.elapsed_time(b) for a, b in zip(starts, ends)))
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    units = m.wet_cells * m.maxl
    value = world * units * args.steps / (total_ms * 1e-3)

    # end to end through the C-ABI: the interval's increments from pinned host memory, the
    # coupling, BIOGEM's ocean tracers and particulates back to pinned host memory
    vd_h = torch.from_numpy(np.ascontiguousarray(st.vdocn)).pin_memory()
    vdb_h = torch.from_numpy(np.ascontiguousarray(st.vdbio_part)).pin_memory()
    vo_h = torch.empty(tuple(st.vocn.shape), dtype=torch.float64).pin_memory()
    vb_h = torch.empty(tuple(st.vbio_part.shape), dtype=torch.float64).pin_memory()
    dp = C.POINTER(C.c_double)
    ptr = lambda t: C.cast(t.data_ptr(), dp)   # noqa: E731
    lib = bg.lib
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for s in range(args.steps):
        lib.gb_bg_set_increments(bg.h, ptr(vd_h), ptr(vdb_h))
        lib.gb_bg_tracercoupling(bg.h, g.h)
        lib.gb_bg_download(bg.h, ptr(vo_h), None, None, ptr(vb_h))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * units * args.steps / e2e_s

    peak, peak_kind = measured_peaks()
    alg = bg_algorithmic_bytes(m.wet_cells, m.maxl, Ls)
    achieved = alg / (total_ms * 1e-3 / args.steps) / 1e9
    if rank == 0:
        line = {
            "metric": "tracer cell-couplings/s", "value": value, "unit": "tracer cell-couplings/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded member and BIOGEM fields, reference grid formulas)",
            "config": {"workload": w["name"], "maxi": m.maxi, "maxj": m.maxj, "maxk": m.maxk, "n_l_ocn": m.maxl,
                       "n_l_sed": Ls, "wet_cells": m.wet_cells,
                       "l2": "not flushed: the fields (2.4 GB) are larger than L2",
                       "parallelism": f"replicas{world}"},
            "e2e": {"value": e2e_value, "unit": "tracer cell-couplings/s",
                    "h2d_bytes_per_step": int(vd_h.numel() + vdb_h.numel()) * 8,
                    "d2h_bytes_per_step": int(vo_h.numel() + vb_h.numel()) * 8,
                    "note": "per coupling: vdocn + vdbio_part H2D (pinned), coupling, vocn + vbio_part D2H"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": profile_traffic("coupling", w["name"]),
                         "peak_source": peak_kind, "kernel": "coupling: k_bg_partials x2, k_bg_seqsum x2, "
                         "k_bg_apply, k_bg_zero, k_bg_halo, step-buffer reload copies",
                         "algorithmic_bytes_per_launch": alg,
                         "note": "algorithmic bytes 8*(6L + 3Ls + 5) per wet cell over the whole coupling"},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            v, n = bg_cpu_rate(m, st)
            line["cpu_baseline"] = {"value": v, "unit": "tracer cell-couplings/s", "cores": 1, "kind": "port",
                                    "sample": f"{n} couplings of the same fields, oracle C restatement, -O2"}
        print(json.dumps(line))
    bg.close()
    g.close()


def _ea_case(w, member: int = 0):
    from cgenie_gb300 import grid, surface
    m = grid.make_member(grid.MemberConfig(maxi=w["maxi"], maxj=w["maxj"], maxk=8, maxl=2, seed=21 + 7919 * member))
    if w.get("kind") == "ice":
        return surface.seaice_case(m, seed=22 + 7919 * member)
    return surface.embm_case(m, seed=22 + 7919 * member)


def _ice_oracle_steps(c, n):
    """n step_seaice steps on the oracles: transport (C restatement), post-processing (NumPy)."""
    from cgenie_gb300 import surface
    from oracle import oracle_lib
    from oracle import surface_np as snp
    p = surface.seaice_post_constants(c)
    for _ in range(n):
        oracle_lib.surface_step(c, 1)
        snp.seaice_post(c.maxk, c.k1, c.tq, c.tq1, c.source, p.rhoio, p.rhoice, p.hlf, p.hmin, p.rdtdim, p.m2mm)


def ea_cpu_rate(case, target_s: float = 10.0):
    """The oracle's tstipa (serial, 1 core): (cell-updates/s, steps)."""
    from cgenie_gb300 import abi
    from oracle import oracle_lib
    c = case.copy()
    run = (lambda k: _ice_oracle_steps(c, k)) if case.kind == abi.GB_EA_SEAICE else \
        (lambda k: oracle_lib.surface_step(c, k))
    t0 = time.perf_counter()
    run(10)
    per = (time.perf_counter() - t0) / 10
    n = max(10, min(100000, int(target_s / max(per, 1e-9))))
    t0 = time.perf_counter()
    run(n)
    dt = time.perf_counter() - t0
    return case.maxi * case.maxj * 2 * n / dt, n


def run_ea(args, rank, world, local, dist):
    """tstipa on one device-resident surface grid: one launch per step."""
    import ctypes as C

    import numpy as np
    import torch
    from cgenie_gb300 import surface
    from cgenie_gb300.goldstein import kernel_launch_count
    w = WORKLOADS[args.workload]
    nmem = w.get("members", 1)
    cases = [_ea_case(w, n) for n in range(nmem)]
    case = cases[0]
    steppers = [surface.SurfaceStepper(c.copy(), device=local) for c in cases]
    for st in steppers:
        st.upload_state()
        st.set_forcing()
    ice = w.get("kind") == "ice"
    if ice:
        for st in steppers:
            st.set_seaice_post(surface.seaice_post_constants(case))
    s = steppers[0]
    step = (lambda: s.step(1)) if nmem == 1 else (lambda: surface.step_many(steppers, 1))
    for _ in range(args.warmup):
        step()
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = kernel_launch_count()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dev_s = time.perf_counter() - t0
    launches = kernel_launch_count() - n0
    clocks = sampler.stop()
    units = case.maxi * case.maxj * 2 * nmem
    value = world * units * args.steps / dev_s
    # end to end: the step's forcing (tqa, uatm, pptn) from pinned host memory, the step, tq back
    src_h = torch.from_numpy(np.ascontiguousarray(case.source)).pin_memory()
    vel_h = torch.from_numpy(np.ascontiguousarray(case.vel)).pin_memory()
    pp_h = None if ice else torch.from_numpy(np.ascontiguousarray(case.pptn)).pin_memory()
    tq_h = torch.empty(tuple(case.tq.shape), dtype=torch.float64).pin_memory()
    fl_h = torch.empty((2, case.maxj, case.maxi), dtype=torch.float64).pin_memory()   # fx_delta, fw_delta
    dp = C.POINTER(C.c_double)
    ptr = lambda t: None if t is None else C.cast(t.data_ptr(), dp)   # noqa: E731
    e2e_steps = args.steps if nmem == 1 else max(1, args.steps // 10)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for st in steppers:
            st.lib.gb_ea_set_forcing(st.h, ptr(src_h), ptr(vel_h), ptr(pp_h))
        step()
        for st in steppers:
            st.lib.gb_ea_download(st.h, ptr(tq_h), None)
            if ice:
                st.lib.gb_ea_download_seaice_fluxes(st.h, ptr(fl_h[0]), ptr(fl_h[1]))
    e2e_s = time.perf_counter() - t0
    peak, peak_kind = measured_peaks()
    # EMBM: read tq, tq1, tqa, uatm (2 each), pptn; write tq, tq1.  Sea ice: the transport reads
    # tq, tq1, dtha, u (2 each) and writes tq, variceth, varicedy; the post-processing reads tq,
    # dtha(1) and writes tq, tq1, fx_delta, fw_delta (23 doubles per cell)
    alg = (23 if ice else 13) * 8 * case.maxi * case.maxj * nmem
    achieved = alg / (dev_s / args.steps) / 1e9
    unit = "ice cell-updates/s" if ice else "air cell-updates/s"
    if rank == 0:
        line = {
            "metric": unit, "value": value, "unit": unit, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded fields on the reference's sin-latitude grid)",
            "config": {"workload": w["name"], "maxi": case.maxi, "maxj": case.maxj, "tracers": 2, "grids": nmem,
                       "timing": "host clock around the synchronous C-ABI step calls (%s each)"
                                 % ("two launches" if ice else "one launch"),
                       "l2": "not flushed: the grid (0.3 MB) lives in L2, as in the model",
                       "parallelism": f"replicas{world}"},
            "e2e": {"value": world * units * e2e_steps / e2e_s, "unit": unit,
                    "h2d_bytes_per_step": int(src_h.numel() + vel_h.numel() + (0 if ice else pp_h.numel())) * 8 * nmem,
                    "d2h_bytes_per_step": int(tq_h.numel() + (fl_h.numel() if ice else 0)) * 8 * nmem,
                    "note": ("per step and grid: dtha + u H2D (pinned), step_seaice, tq + fx_delta + fw_delta D2H"
                             if ice else "per step and grid: tqa + uatm + pptn H2D (pinned), step, tq D2H")},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": peak_kind,
                         "kernel": "k_surface_step + k_seaice_post (one step)" if ice else "k_surface_step",
                         "algorithmic_bytes_per_launch": alg,
                         "note": "latency-bound: one cluster of 8 blocks per tracer, 5 cluster-barrier-separated "
                                 "sweeps per step; the HBM roofline does not bind a 0.3 MB grid"},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            v, n = ea_cpu_rate(case)
            line["cpu_baseline"] = {"value": v, "unit": unit, "cores": 1, "kind": "port",
                                    "sample": f"{n} steps of the same grid, oracle C restatement, -O2"
                                              + (" + NumPy post-processing" if ice else "")}
        print(json.dumps(line))
    for st in steppers:
        st.close()


def _mo_member(w):
    from cgenie_gb300 import grid, momentum
    m = grid.make_member(grid.MemberConfig(maxi=w["maxi"], maxj=w["maxj"], maxk=w["maxk"], maxl=2, seed=31,
                                           mask="basin_island"))
    return m, momentum.make_case(m, seed=32)


def mo_cpu_rate(m, case, target_s: float = 10.0):
    """The oracle's momentum step (serial, 1 core): (wet-cell updates/s, steps)."""
    from oracle import oracle_lib
    o = oracle_lib.OracleMomentum(case)
    t0 = time.perf_counter()
    o.step(m.rho)
    per = time.perf_counter() - t0
    n = max(3, min(20000, int(target_s / max(per, 1e-9))))
    t0 = time.perf_counter()
    for _ in range(n):
        o.step(m.rho)
    dt = time.perf_counter() - t0
    o.close()
    return m.wet_cells * n / dt, n


def run_mo(args, rank, world, local, dist):
    """The momentum step on one basin: device-resident timing (CUDA events on the ocean
    handle's stream), end to end with the wind uploaded and u read back."""
    import ctypes as C

    import numpy as np
    import torch
    from cgenie_gb300 import momentum
    from cgenie_gb300.goldstein import kernel_launch_count, new_member_run
    w = WORKLOADS[args.workload]
    m, case = _mo_member(w)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g = new_member_run(m, device=local, stream=stream.cuda_stream)
    mo = momentum.Momentum(case, device=local)
    mo.set_wind()
    for _ in range(args.warmup):
        mo.step(g)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = kernel_launch_count()
    for s_ in range(args.steps):
        starts[s_].record(stream)
        mo.step(g)
        ends[s_].record(stream)
    torch.cuda.synchronize()
    launches = kernel_launch_count() - n0
    clocks = sampler.stop()
    total_ms = float(sum(a.elapsed_time(b) for a, b in zip(starts, ends)))
    units = m.wet_cells
    value = world * units * args.steps / (total_ms * 1e-3)
    tau_h = torch.from_numpy(np.ascontiguousarray(case.tau)).pin_memory()
    dzt_h = torch.from_numpy(np.ascontiguousarray(case.dztau)).pin_memory()
    dzv_h = torch.from_numpy(np.ascontiguousarray(case.dztav)).pin_memory()
    u_h = torch.empty((case.maxk, case.maxj + 1, case.maxi + 1, 3), dtype=torch.float64).pin_memory()
    dp = C.POINTER(C.c_double)
    ptr = lambda t: C.cast(t.data_ptr(), dp)   # noqa: E731
    t0 = time.perf_counter()
    for _ in range(args.steps):
        mo.lib.gb_mo_set_wind(mo.h, ptr(tau_h), ptr(dzt_h), ptr(dzv_h))
        mo.lib.gb_mo_step(mo.h, g.h)
        mo.lib.gb_mo_download(mo.h, ptr(u_h), None, None, None)
    e2e_s = time.perf_counter() - t0
    peak, peak_kind = measured_peaks()
    nm = case.maxi * (case.maxj + 1)
    alg = 8 * nm * nm   # the streamfunction product reads the inverse once
    achieved = alg / (total_ms * 1e-3 / args.steps) / 1e9
    if rank == 0:
        line = {
            "metric": "wet-cell momentum updates/s", "value": value, "unit": "wet-cell momentum updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded basin with two islands, reference grid formulas)",
            "config": {"workload": w["name"], "maxi": case.maxi, "maxj": case.maxj, "maxk": case.maxk,
                       "isles": case.isles, "wet_cells": m.wet_cells,
                       "l2": "not flushed: the 14 MB inverse and the fields stay in L2, as between model steps",
                       "parallelism": f"replicas{world}"},
            "e2e": {"value": world * units * args.steps / e2e_s, "unit": "wet-cell momentum updates/s",
                    "h2d_bytes_per_step": int(tau_h.numel() + dzt_h.numel() + dzv_h.numel()) * 8,
                    "d2h_bytes_per_step": int(u_h.numel()) * 8,
                    "note": "per step: the wind stress H2D (pinned), momentum step, u D2H"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": peak_kind, "kernel": "momentum step (8 kernels)",
                         "algorithmic_bytes_per_launch": alg,
                         "note": "latency-bound chain of 8 small kernels; the inverse (8*nm^2 bytes) is the "
                                 "largest read"},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            v, n = mo_cpu_rate(m, case)
            line["cpu_baseline"] = {"value": v, "unit": "wet-cell momentum updates/s", "cores": 1, "kind": "port",
                                    "sample": f"{n} steps of the same basin, oracle C restatement (banded LU), -O2"}
        print(json.dumps(line))
    mo.close()
    g.close()


def _rs_coords(m):
    import numpy as np
    return (np.linspace(0.0, 360.0, m.maxi, endpoint=False) + 0.5, np.linspace(-89.5, 89.5, m.maxj),
            np.cumsum(np.linspace(10.0, 400.0, m.maxk)))


def rs_cpu_rate(m, target_s: float):
    """The reference's restart path restated on the host: outm_netcdf's field forming (NumPy
    restatement of the oracle) and a netCDF classic write (scipy's writer standing in for the
    netCDF library), repeated for about target_s seconds."""
    import tempfile

    import numpy as np
    from scipy.io import netcdf_file
    from oracle import restart_np
    lon, lat, ncdepth = _rs_coords(m)
    n, t0 = 0, time.perf_counter()
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "goldstein_restart.nc")
        while True:
            f = restart_np.restart_fields(m.ts, m.u, m.k1, m.maxi, m.maxj, m.maxk)
            with netcdf_file(path, "w", version=1) as nc:
                for d, ln in (("nrecs", 1), ("longitude", m.maxi), ("latitude", m.maxj), ("depth", m.maxk)):
                    nc.createDimension(d, ln)
                for v, a, d in (("longitude", lon, "longitude"), ("latitude", lat, "latitude")):
                    nc.createVariable(v, "f", (d,))[:] = a
                nc.createVariable("depth", "f", ("depth",))[:] = restart_np.depths1(ncdepth)
                for v in ("ioffset", "iyear", "imonth", "iday"):
                    nc.createVariable(v, "i", ("nrecs",))[:] = 1
                for v, a in zip(("temp", "salinity", "uvel", "vvel"), f):
                    nc.createVariable(v, "d", ("depth", "latitude", "longitude"))[:] = a
                for v in ("evap", "late", "sens"):
                    nc.createVariable(v, "d", ("latitude", "longitude"))[:] = np.zeros((m.maxj, m.maxi))
            n += 1
            dt = time.perf_counter() - t0
            if dt >= target_s or n >= 200:
                break
    return n * m.maxi * m.maxj * m.maxk / dt, n


def run_rs(args, rank, world, local, dist):
    """Restart writes of a device-resident ocean (outm_netcdf): the fields formed on the device
    in the file's byte order and one D2H copy.  value: ocean cells per second of that device
    part (gb_rs_pack_goldstein + the copy into pinned memory, CUDA events), the state resident;
    e2e: the public call gb_rs_write_goldstein, file written, timed on the host clock."""
    import tempfile

    import torch
    from cgenie_gb300 import grid, restart
    from cgenie_gb300.goldstein import kernel_launch_count, new_member_run
    import dataclasses
    w = WORKLOADS[args.workload]
    m = grid.make_member(dataclasses.replace(getattr(grid, w["factory"])(), **({"maxl": w["maxl"]} if "maxl" in w else {})))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g = new_member_run(m, device=local, stream=stream.cuda_stream)
    g.tstepo(1)
    lon, lat, ncdepth = _rs_coords(m)
    cal = restart.Calendar(iyear=2000, imonth=1, day=1.0)
    td = tempfile.mkdtemp(prefix="gb_rs_")
    path = os.path.join(td, f"goldstein_restart_r{rank}.nc")
    cells = m.maxi * m.maxj * m.maxk
    dev = torch.empty(4 * cells, dtype=torch.float64, device=f"cuda:{local}")
    host = torch.empty(4 * cells, dtype=torch.float64).pin_memory()
    for _ in range(args.warmup):
        restart.pack_goldstein(g, dev.data_ptr())
        host.copy_(dev, non_blocking=True)
        restart.write_goldstein(g, path, cal, lon, lat, ncdepth)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    flush = torch.empty(64 << 20, dtype=torch.float32, device=f"cuda:{local}")   # 256 MB > L2
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = kernel_launch_count()
    for s_ in range(args.steps):
        flush.zero_()
        ev[s_][0].record(stream)
        restart.pack_goldstein(g, dev.data_ptr())
        ev[s_][1].record(stream)
        host.copy_(dev, non_blocking=True)
        ev[s_][2].record(stream)
    torch.cuda.synchronize()
    launches = kernel_launch_count() - n0
    clocks = sampler.stop()
    kern_ms = float(sum(e[0].elapsed_time(e[1]) for e in ev)) / args.steps
    dev_ms = float(sum(e[0].elapsed_time(e[2]) for e in ev)) / args.steps
    t1 = time.perf_counter()
    for _ in range(args.steps):
        restart.write_goldstein(g, path, cal, lon, lat, ncdepth)
    e2e_s = time.perf_counter() - t1
    size = os.path.getsize(path)
    os.remove(path)
    os.rmdir(td)
    cells = m.maxi * m.maxj * m.maxk
    peak, peak_kind = measured_peaks()
    alg = 64 * cells   # per cell: T, S and u, v read (32 B), the four fields written (32 B)
    if rank == 0:
        line = {
            "metric": "ocean cells written/s", "value": world * cells / (dev_ms * 1e-3), "unit": "ocean cells written/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": f"synthetic (seeded 360x180x32 ocean, {m.maxl} tracers, one step taken)",
            "config": {"workload": w["name"], "maxi": m.maxi, "maxj": m.maxj, "maxk": m.maxk, "maxl": m.maxl,
                       "file_bytes": size, "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas{world}"},
            "e2e": {"value": world * cells * args.steps / e2e_s, "unit": "ocean cells written/s",
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 32 * cells,
                    "note": "per step: gb_rs_write_goldstein, the public call: device fields, one D2H into the "
                            "pinned file image, the file written (page cache)"},
            "roofline": {"bound": "hbm", "achieved": alg / (kern_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / (kern_ms * 1e-3) / 1e9 / peak, "traffic": None, "peak_source": peak_kind,
                         "kernel": "k_rs_pack (stream events around gb_rs_pack_goldstein)", "kernel_us": 1e3 * kern_ms,
                         "algorithmic_bytes_per_launch": alg},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            v, n = rs_cpu_rate(m, target_s=10.0)
            line["cpu_baseline"] = {"value": v, "unit": "ocean cells written/s", "cores": 1, "kind": "port",
                                    "sample": f"{n} restarts of the same ocean: NumPy field forming + scipy netCDF write"}
        print(json.dumps(line))
    g.close()


def run_ocean(args, rank, world, local, dist):
    """Momentum + tracer step + BIOGEM coupling on one basin, all on the device."""
    import torch
    from cgenie_gb300 import abi, biogem, grid, momentum
    from cgenie_gb300.goldstein import kernel_launch_count, new_member_run
    w = WORKLOADS[args.workload]
    m = grid.make_member(grid.MemberConfig(maxi=w["maxi"], maxj=w["maxj"], maxk=w["maxk"], maxl=w["maxl"], seed=41,
                                           mask="basin_island", tracer_kind="bgc", **w.get("member_kw", {})))
    case = momentum.make_case(m, seed=42)
    st = biogem.make_state(m, n_l_sed=4, seed=43)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g = new_member_run(m, device=local, stream=stream.cuda_stream, precision=abi.GB_GO_FP32FLUX)
    mo = momentum.Momentum(case, device=local)
    mo.set_wind()
    bg = biogem.BiogemCoupling(m, n_l_sed=4, device=local)
    bg.upload(st)
    bg.set_increments(st)
    every = w["couple_every"]

    def ocean_step(n):
        mo.step(g)
        g.tstepo(1)
        if (n + 1) % every == 0:
            bg.tracercoupling(g)

    for n in range(args.warmup):
        ocean_step(n)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    n0 = kernel_launch_count()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for n in range(args.steps):
        ocean_step(n)
    end.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = kernel_launch_count() - n0
    total_ms = start.elapsed_time(end)
    units = m.wet_cells * m.maxl
    value = world * units * args.steps / (total_ms * 1e-3)
    peak, peak_kind = measured_peaks()
    alg = algorithmic_bytes(m)
    if rank == 0:
        line = {
            "metric": "tracer cell-updates/s", "value": value, "unit": "tracer cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 transfers, f64 state",
            "data": "synthetic (seeded basin with two islands, BIOGEM fields, reference grid formulas)",
            "config": {"workload": w["name"], "maxi": m.maxi, "maxj": m.maxj, "maxk": m.maxk, "maxl": m.maxl,
                       "wet_cells": m.wet_cells, "couple_every": every, "precision": "fp32flux",
                       "l2": "not flushed: the whole model state stays on the device, as in a run",
                       "parallelism": f"replicas{world}"},
            "e2e": {"value": value, "unit": "tracer cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "note": "the ocean step moves nothing across the host boundary: rho, u, ts stay on the device"},
            "roofline": {"bound": "hbm", "achieved": alg / (total_ms * 1e-3 / args.steps) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": alg / (total_ms * 1e-3 / args.steps) / 1e9 / peak, "traffic": None,
                         "peak_source": peak_kind, "kernel": "ocean step (momentum graph, tracer step, coupling)",
                         "algorithmic_bytes_per_launch": alg, "note": "tracer-step algorithmic bytes per ocean step"},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            v, n, _ = ocean_cpu_rate(w, w.get("cpu_steps", 20))
            line["cpu_baseline"] = {"value": v, "unit": "tracer cell-updates/s", "cores": 1, "kind": "port",
                                    "sample": f"{n} ocean steps (momentum, tracer step, coupling), oracle C "
                                              f"restatements, serial"}
        print(json.dumps(line))
    bg.close()
    mo.close()
    g.close()


def ocean_cpu_rate(w, steps):
    """The oracles' ocean step (momentum, tracer step, coupling every few steps), serial."""
    import numpy as np
    from cgenie_gb300 import biogem, grid, momentum
    from oracle import oracle_lib
    m = grid.make_member(grid.MemberConfig(maxi=w["maxi"], maxj=w["maxj"], maxk=w["maxk"], maxl=w["maxl"], seed=41,
                                           mask="basin_island", tracer_kind="bgc", **w.get("member_kw", {})))
    case = momentum.make_case(m, seed=42)
    st = biogem.make_state(m, n_l_sed=4, seed=43)
    om = oracle_lib.OracleMomentum(case)
    s = oracle_lib.OracleState(m)
    t0 = time.perf_counter()
    for n in range(steps):
        om.step(s.rho)
        s.u = np.ascontiguousarray(om.state()["u"])
        s.step(1)
        if (n + 1) % w["couple_every"] == 0:
            go, go1 = oracle_lib.bg_tracercoupling(m, st, oracle_lib.go_ts_interior(s.ts))
            oracle_lib.after_coupling(s, go, go1)
    dt = time.perf_counter() - t0
    om.close()
    return m.wet_cells * m.maxl * steps / dt, steps, dt


def run_reference(args, rank, world):
    w = dict(WORKLOADS[args.workload])
    if args.workload in ("ocean36", "ocean5"):
        v, n, dt = ocean_cpu_rate(w, w.get("cpu_steps", max(5, min(args.steps, 50))))
        line = {
            "metric": "tracer cell-updates/s", "value": v, "unit": "tracer cell-updates/s", "impl": "reference",
            "n_gpus": world, "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * dt / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"], "couple_every": w["couple_every"]},
            "cpu_baseline": {"value": v, "unit": "tracer cell-updates/s", "cores": 1, "kind": "port",
                             "sample": f"{n} ocean steps (momentum, tracer step, coupling), oracle C restatements, serial"},
            "e2e": {"value": v, "unit": "tracer cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    if args.workload in ("rs5", "rs5s"):
        import dataclasses
        from cgenie_gb300 import grid
        m = grid.make_member(dataclasses.replace(getattr(grid, w["factory"])(), **({"maxl": w["maxl"]} if "maxl" in w else {})))
        v, n = rs_cpu_rate(m, target_s=min(20.0, 2.0 * max(args.steps, 1)))
        line = {
            "metric": "ocean cells written/s", "value": v, "unit": "ocean cells written/s", "impl": "reference",
            "n_gpus": world, "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * m.maxi * m.maxj * m.maxk / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"], "maxi": m.maxi, "maxj": m.maxj, "maxk": m.maxk, "maxl": m.maxl},
            "cpu_baseline": {"value": v, "unit": "ocean cells written/s", "cores": 1, "kind": "port",
                             "sample": f"{n} restarts: NumPy restatement of outm_netcdf's fields + scipy netCDF write"},
            "e2e": {"value": v, "unit": "ocean cells written/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    if args.workload == "mo36":
        m, case = _mo_member(w)
        v, n = mo_cpu_rate(m, case, target_s=min(10.0, 0.01 * max(args.steps, 1)))
        line = {
            "metric": "wet-cell momentum updates/s", "value": v, "unit": "wet-cell momentum updates/s",
            "impl": "reference", "n_gpus": world, "steps": n, "warmup": args.warmup,
            "ms_per_step": 1e3 * m.wet_cells / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"], "maxi": case.maxi, "maxj": case.maxj, "maxk": case.maxk, "isles": case.isles},
            "cpu_baseline": {"value": v, "unit": "wet-cell momentum updates/s", "cores": 1, "kind": "port",
                             "sample": f"{n} steps, oracle C restatement, serial (the reference routine is serial)"},
            "e2e": {"value": v, "unit": "wet-cell momentum updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    if args.workload in ("ea64", "ea36e", "ice64"):
        case = _ea_case(w)
        v, n = ea_cpu_rate(case, target_s=min(10.0, 0.01 * max(args.steps, 1)))
        unit = "ice cell-updates/s" if w.get("kind") == "ice" else "air cell-updates/s"
        line = {
            "metric": unit, "value": v, "unit": unit, "impl": "reference",
            "n_gpus": world, "steps": n, "warmup": args.warmup, "ms_per_step": 1e3 * case.maxi * case.maxj * 2 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"], "maxi": case.maxi, "maxj": case.maxj, "tracers": 2},
            "cpu_baseline": {"value": v, "unit": unit, "cores": 1, "kind": "port",
                             "sample": f"{n} steps, oracle C restatement" + (" + NumPy post-processing" if w.get("kind") == "ice" else "")
                                       + ", serial (the reference routine is serial)"},
            "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    if args.workload == "bg5":
        from cgenie_gb300 import biogem, grid
        m = grid.make_member(getattr(grid, w["factory"])())
        st = biogem.make_state(m, n_l_sed=w["n_l_sed"], seed=5)
        from oracle import oracle_lib
        go = oracle_lib.go_ts_interior(m.ts)
        for _ in range(min(args.warmup, 1)):
            go, _ = oracle_lib.bg_tracercoupling(m, st, go)
        steps = max(1, min(args.steps, 10))
        t0 = time.perf_counter()
        for _ in range(steps):
            go, _ = oracle_lib.bg_tracercoupling(m, st, go)   # successive couplings of the evolving fields
        dt = time.perf_counter() - t0
        value = m.wet_cells * m.maxl * steps / dt
        line = {
            "metric": "tracer cell-couplings/s", "value": value, "unit": "tracer cell-couplings/s",
            "impl": "reference", "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"], "n_l_ocn": m.maxl, "n_l_sed": w["n_l_sed"], "wet_cells": m.wet_cells},
            "cpu_baseline": {"value": value, "unit": "tracer cell-couplings/s", "cores": 1, "kind": "port",
                             "sample": f"{steps} couplings (of {args.steps} asked), oracle C restatement, serial "
                                       f"(the reference routine is serial)"},
            "e2e": {"value": value, "unit": "tracer cell-couplings/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    if args.workload == "c3" and args.members:
        w["members"] = args.members
    if args.workload == "c3":
        value, cores, cu_step = oracle_pool_rate(w["members"], w["seed"], args.warmup, args.steps, faithful=True)
        line = {
            "metric": "tracer cell-updates/s", "value": value, "unit": "tracer cell-updates/s", "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * cu_step / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["name"], "members": w["members"], "seed": w["seed"]},
            "cpu_baseline": {"value": value, "unit": "tracer cell-updates/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} timed steps of all {w['members']} members, oracle C restatement "
                                       f"with the reference's dead copies, one process per core"},
            "e2e": {"value": value, "unit": "tracer cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    from cgenie_gb300 import grid
    m = grid.make_member(getattr(grid, w["factory"])())
    from oracle import oracle_lib
    s = oracle_lib.OracleState(m)
    for _ in range(args.warmup):
        s.step(1, faithful=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.step(1, faithful=True)
    dt = time.perf_counter() - t0
    value = m.wet_cells * m.maxl * args.steps / dt
    line = {
        "metric": "tracer cell-updates/s", "value": value, "unit": "tracer cell-updates/s", "impl": "reference",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w["name"], "maxi": m.maxi, "maxj": m.maxj, "maxk": m.maxk, "maxl": m.maxl,
                   "wet_cells": m.wet_cells, "diso": bool(m.cfg.diso)},
        "cpu_baseline": {"value": value, "unit": "tracer cell-updates/s", "cores": 1, "kind": "port",
                         "sample": f"{args.steps} timed steps of the workload member, serial (the reference is serial)"},
        "e2e": {"value": value, "unit": "tracer cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def _tracer_errs(m, a, b):
    """Per-tracer error max|a - b| / max|b| over the wet interior cells."""
    import numpy as np
    kk = np.arange(m.maxk + 2)[:, None, None]
    wet = (kk >= m.k1[None]) & (kk >= 1) & (kk <= m.maxk)
    wet[:, 0, :] = wet[:, -1, :] = False
    wet[:, :, 0] = wet[:, :, -1] = False
    out = []
    for l in range(m.maxl):
        x, y = a[..., l][wet], b[..., l][wet]
        out.append(float(np.max(np.abs(x - y)) / max(float(np.max(np.abs(y))), 1e-300)))
    return out


def run_c3(args, rank, world, local, dist):
    import numpy as np
    import torch
    from cgenie_gb300.ensemble import Ensemble
    from cgenie_gb300.goldstein import kernel_launch_count, new_member_run
    from cgenie_gb300.replicas import job_time, job_units, partition

    w = dict(WORKLOADS["c3"])
    if args.members:
        w["members"] = args.members
        w["name"] = w["name"].replace("ensemble256", f"ensemble{args.members}")
    # one ensemble of members x ranks, partitioned: rank r advances members r::world (weak
    # scaling, no collective on the data path); at one rank it is the workload's ensemble
    from cgenie_gb300 import grid as _g
    cfgs_all = _g.ensemble_configs(w["members"] * world, seed=w["seed"])
    mems = [_g.make_member(cfgs_all[i]) for i in partition(len(cfgs_all), rank, world)]
    cu_step = sum(m.wet_cells * m.maxl for m in mems)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ens = Ensemble(device=local, use_graph=True, stream=stream.cuda_stream)
    ids = ens.add_many(mems)
    if args.steps_before:
        ens.step(args.steps_before)
    for _ in range(args.warmup):
        ens.step(1)
    torch.cuda.synchronize()

    # ---- device-resident timing: one graph replay (a full step of all members) per step
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = kernel_launch_count()
    for k in range(args.steps):
        starts[k].record(stream)
        ens.step(1)
        ends[k].record(stream)
    torch.cuda.synchronize()
    launches = kernel_launch_count() - n0
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = 1e3 * job_time(1e-3 * float(sum(ms)), dist, "cuda")
    all_cu_step = job_units(cu_step, dist, "cuda")
    value = all_cu_step * args.steps / (total_ms * 1e-3)
    done = args.steps_before + args.warmup + args.steps

    # ---- error against the FP64 path (bit-identical to the FP64 oracle) after at least the
    # configuration's 1000 steps, per tracer, on a sample of the members (per grid shape the
    # fewest, the most and a middle tracer count)
    from cgenie_gb300 import grid as _grid
    err_steps = max(done, args.err_steps) if args.err_steps > 0 else done
    if err_steps > done:
        ens.step(err_steps - done)
    sample = _grid.error_sample([m.cfg for m in mems]) if args.err_steps > 0 else []
    per_tracer = [0.0] * max(m.maxl for m in mems)
    for i in sample:
        out = ens.download(ids[i])
        g = new_member_run(mems[i], device=local, stream=stream.cuda_stream)
        g.tstepo(err_steps)
        ref = g.download()
        g.close()
        for l, e in enumerate(_tracer_errs(mems[i], out["ts"], ref["ts"])):
            per_tracer[l] = max(per_tracer[l], e)
    err = max(per_tracer) if sample else None
    ens.close()

    # ---- the plain per-member GPU path (FP64 drop-in, one member at a time), two of each shape
    plain_cu, plain_s = 0, 0.0
    for i in range(6):
        g = new_member_run(mems[i], device=local, stream=stream.cuda_stream)
        g.tstepo(2)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        g.tstepo(20)
        b.record(stream)
        torch.cuda.synchronize()
        plain_s += a.elapsed_time(b) * 1e-3
        plain_cu += mems[i].wet_cells * mems[i].maxl * 20
        g.close()
    plain_value = plain_cu / plain_s

    # ---- end to end through the C-ABI: admit from mapped pinned host arrays (gb_ens_host_alloc),
    # step, download every member into such arrays (the host buffers exist before the timed region)
    import dataclasses
    from cgenie_gb300.ensemble import host_copy
    hmems = [dataclasses.replace(m, ts=host_copy(m.ts), u=host_copy(m.u)) for m in mems]
    houts = [dict(ts=host_copy(np.zeros_like(m.ts)), rho=host_copy(np.zeros_like(m.rho)),
                  cost=host_copy(np.zeros_like(m.cost))) for m in mems]
    def e2e_job():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        e2 = Ensemble(device=local, use_graph=True, stream=stream.cuda_stream)
        ids2 = e2.add_many(hmems)
        t1 = time.perf_counter()
        e2.step(args.steps)
        e2.sync()
        t2 = time.perf_counter()
        outs = e2.download_many(ids2, out=houts)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        e2.close()
        return t0, t1, t2, t3, outs

    # one untimed job first (first-use costs of the mapped buffers and the memory pool), then
    # the timed job: the whole sequence again from a new ensemble
    e2e_job()
    t0, t1, t2, t3, outs = e2e_job()
    e2e_s = job_time(t3 - t0, dist, "cuda")
    e2e_parts = {"admit_s": round(t1 - t0, 5), "steps_s": round(t2 - t1, 5), "download_s": round(t3 - t2, 5)}
    e2e_value = all_cu_step * args.steps / e2e_s
    h2d = sum(m.ts.nbytes + m.u.nbytes for m in mems) / args.steps
    d2h = sum(o["ts"].nbytes + o["rho"].nbytes + o["cost"].nbytes for o in outs) / args.steps

    # ---- serving (the serving configuration at a bounded request count): Poisson arrivals at
    # 50 runs/s of 200-5000-step members of the three grids, admitted by free HBM, continuously
    # batched; p50/p99 run latency and tracer cell-updates per second of wall time
    serving = None
    if args.serving_requests > 0 and rank == 0:
        from cgenie_gb300.serving import Server, poisson_requests
        reqs = poisson_requests(args.serving_requests, rate=50.0, seed=7)
        srv = Server(chunk=25, device=local)
        st = srv.run(reqs)
        srv.close()
        serving = {"requests": st["requests"], "arrival_rate_per_s": 50.0, "steps_range": [200, 5000],
                   "p50_latency_s": st["p50_latency_s"], "p99_latency_s": st["p99_latency_s"],
                   "cell_updates_per_s": st["cell_updates_per_s"], "wall_s": st["wall_s"],
                   "gpu_busy_over_wall": st["busy_s"] / st["wall_s"] if st["wall_s"] > 0 else None,
                   "max_active": st["max_active"],
                   "note": "wall time is set by the arrivals (the last arrives at ~requests/rate s); "
                           "busy = time in the batched steps"}

    peak, peak_kind = measured_peaks()
    alg = sum(algorithmic_bytes(m) for m in mems)
    achieved = alg / (total_ms * 1e-3 / args.steps) / 1e9
    traffic = profile_traffic("k_step_fp32", w["name"])
    l2_bytes = profile_traffic("l2_bytes_transfer_kernels", w["name"])
    if rank == 0:
        line = {
            "metric": "tracer cell-updates/s", "value": value, "unit": "tracer cell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 transfers, f64 state",
            "data": "synthetic (seeded members, reference grid formulas)",
            "config": {"workload": w["name"], "members": w["members"], "seed": w["seed"],
                       "cell_updates_per_step": all_cu_step, "precision": "fp32flux",
                       "l2": "not flushed: the resident states (2 x 0.6 GB) exceed L2",
                       "cuda_graph": True, "parallelism": f"one ensemble of {w['members'] * world} members partitioned over {world} rank(s) "
                                      "(members r::N), no collective on the data path",
                       "plain_per_member_gpu": plain_value, "batched_over_plain": value / plain_value,
                       "max_rel_err_vs_fp64": err, "err_after_steps": err_steps, "err_members": len(sample),
                       "per_tracer_err": [float(f"{e:.3e}") for e in per_tracer],
                       "err_note": "per tracer index: max over the sampled members of max|x - x_fp64| / max|x_fp64| "
                                   "over wet cells, against each member's FP64 run (the reference arithmetic)"},
            "e2e": {"value": e2e_value, "unit": "tracer cell-updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "parts": e2e_parts,
                    "note": f"whole job through the C-ABI: admit {w['members']} members from mapped pinned host arrays, "
                            f"{args.steps} steps, download every member into mapped pinned host arrays; the "
                            f"second of two identical jobs (the first absorbs first-use costs)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "batched step: k_step_fp32 (T-S and tracer-group instances) + k_co_decide + k_co_mix + k_rescale",
                         "algorithmic_bytes_per_launch": alg,
                         "note": "achieved = algorithmic bytes of a step (16 L + 24 per wet cell, k1) / step time",
                         "l2": None if l2_bytes is None else {
                             "bytes_per_step": l2_bytes, "gbs": l2_bytes / (total_ms * 1e-3 / args.steps) / 1e9,
                             "note": "L2 traffic of the two transfer kernels per step (ncu, 64-member capture scaled "
                                     "to this ensemble) over the measured step time"}},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if serving is not None:
            line["serving"] = serving
        if not args.no_cpu_baseline:
            cpu, cores, _ = oracle_pool_rate(w["members"], w["seed"], 1, 12, faithful=True)
            line["cpu_baseline"] = {"value": cpu, "unit": "tracer cell-updates/s", "cores": cores, "kind": "port",
                                    "sample": f"12 steps of all {w['members']} members, oracle C restatement with "
                                              "the reference's dead copies, one process per core"}
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c3", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serving-requests", type=int, default=1000,
                    help="c3: requests of the serving leg (Poisson, 50/s; 0: no serving leg)")
    ap.add_argument("--err-steps", type=int, default=1000,
                    help="c3: steps after which the per-tracer error against the FP64 path is taken (0: no error leg)")
    ap.add_argument("--members", type=int, default=0, help="c3: members of the ensemble (default 256)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32flux"], help="single-grid workloads")
    ap.add_argument("--steps-before", type=int, default=0,
                    help="c3: steps taken before the warm-up (the members' convection develops over time)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, rank, world)
        return

    import numpy as np
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from cgenie_gb300 import build, grid
    build.build()
    from cgenie_gb300.goldstein import kernel_launch_count, new_member_run
    if args.workload == "c3":
        run_c3(args, rank, world, local, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in ("ocean36", "ocean5"):
        run_ocean(args, rank, world, local, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in ("rs5", "rs5s"):
        run_rs(args, rank, world, local, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload == "mo36":
        run_mo(args, rank, world, local, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in ("ea64", "ea36e", "ice64"):
        run_ea(args, rank, world, local, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload == "bg5":
        run_bg(args, rank, world, local, dist)
        if dist:
            dist.destroy_process_group()
        return

    w = WORKLOADS[args.workload]
    m = grid.make_member(getattr(grid, w["factory"])())
    # a dedicated stream: the legacy default stream's handle is 0, which the C-ABI
    # reads as "the handle's own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    from cgenie_gb300 import abi
    prec = abi.GB_GO_FP32FLUX if args.precision == "fp32flux" else abi.GB_GO_FP64
    g = new_member_run(m, device=local, stream=stream.cuda_stream, precision=prec)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        g.tstepo(1)
    torch.cuda.synchronize()

    # ---- device-resident timing (L2 flushed before every step)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = kernel_launch_count()
    for s in range(args.steps):
        flush.fill_(float(s))
        starts[s].record(stream)
        g.tstepo(1)
        ends[s].record(stream)
    torch.cuda.synchronize()
    launches = kernel_launch_count() - n0
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = float(sum(ms))
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    cu_per_step = m.wet_cells * m.maxl
    value = world * cu_per_step * args.steps / (total_ms * 1e-3)

    # ---- end to end through the C-ABI with host buffers
    NI, NJ = m.maxi + 2, m.maxj + 2
    top_h = torch.zeros((NJ, NI, m.maxl), dtype=torch.float64).pin_memory()
    u_h = torch.from_numpy(np.ascontiguousarray(m.u)).pin_memory()
    rho_h = torch.empty(tuple(m.rho.shape), dtype=torch.float64).pin_memory()
    import ctypes as C
    lib = g.lib
    dp = C.POINTER(C.c_double)
    top_p = C.cast(top_h.data_ptr(), dp)
    u_p = C.cast(u_h.data_ptr(), dp)
    rho_p = C.cast(rho_h.data_ptr(), dp)
    e2e_steps = args.steps
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        lib.gb_go_set_forcing(g.h, top_p)
        lib.gb_go_set_velocity(g.h, u_p)
        lib.gb_go_tstepo(g.h, 1)
        lib.gb_go_download(g.h, None, None, rho_p, None, None, None, None)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * cu_per_step * e2e_steps / e2e_s
    h2d = top_h.numel() * 8 + u_h.numel() * 8
    d2h = rho_h.numel() * 8

    # ---- roofline of the dominant kernel (the step kernel is the only launch per step)
    peak, peak_kind = measured_peaks()
    alg = algorithmic_bytes(m)
    avg_s = total_ms * 1e-3 / args.steps
    achieved = alg / avg_s / 1e9
    kname = "k_step_fp32" if args.precision == "fp32flux" else "k_step_fp64"
    traffic = profile_traffic(kname, w["name"])

    if rank == 0:
        line = {
            "metric": "tracer cell-updates/s", "value": value, "unit": "tracer cell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 transfers, f64 state" if args.precision == "fp32flux" else "f64",
            "data": "synthetic (seeded member, reference grid formulas)",
            "config": {"workload": w["name"], "maxi": m.maxi, "maxj": m.maxj, "maxk": m.maxk, "maxl": m.maxl,
                       "wet_cells": m.wet_cells, "diso": bool(m.cfg.diso),
                       "precision": "fp32flux" if args.precision == "fp32flux" else "fp64 plain",
                       "l2": "flushed before every timed step", "parallelism": f"replicas{world}"},
            "e2e": {"value": e2e_value, "unit": "tracer cell-updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "note": "per step: forcing + u H2D (pinned), step, rho D2H; L2 not flushed"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": kname, "algorithmic_bytes_per_launch": alg,
                         "note": ("split-precision form on one grid: the batched kernels with one member"
                                  if args.precision == "fp32flux" else
                                  "the plain FP64 form is bound by the FP64 issue rate on GB300, not by HBM")},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(m)
        print(json.dumps(line))
    g.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
