"""Benchmark of the GB300 GOLDSTEIN tracer step (one JSON line on rank 0).

Workloads (seeded synthetic members with the reference's grid formulas):
  c2  single member 36x36x16, 17 tracers, isoneutral branch on, FP64 plain form
  c1  single member 36x36x16, 2 tracers, FP64 plain form

A step is one tracer timestep (tstepo) of the member.  `value` is tracer
cell-updates/s with the state resident in HBM; `e2e` is the same metric through
the C-ABI with host buffers: every step uploads the surface forcing and the
velocities from pinned host memory and reads rho back (the per-step exchange
with the momentum solver, goldstein.f90:167-170,176-177,443-450 minus the state
copies that residency removes).  The state (~3.5 MB) fits in L2, so L2 is
flushed (a 256 MB write) before every timed step and the step is timed alone
with CUDA events on the library's stream.

--impl reference times the reference algorithm on the host cores instead (the
oracle's C restatement of goldstein.f90:2280-2842, serial like the reference).
Multi-GPU (torchrun): every rank runs an independent replica (members are
independent), weak scaling, time = max over ranks.
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
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

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
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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


def run_reference(args, rank, world):
    from cgenie_gb300 import grid
    w = WORKLOADS[args.workload]
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
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

    w = WORKLOADS[args.workload]
    m = grid.make_member(getattr(grid, w["factory"])())
    # a dedicated stream: the legacy default stream's handle is 0, which the C-ABI
    # reads as "the handle's own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g = new_member_run(m, device=local, stream=stream.cuda_stream)
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
    traffic = profile_traffic("k_step_fp64", w["name"])

    if rank == 0:
        line = {
            "metric": "tracer cell-updates/s", "value": value, "unit": "tracer cell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded member, reference grid formulas)",
            "config": {"workload": w["name"], "maxi": m.maxi, "maxj": m.maxj, "maxk": m.maxk, "maxl": m.maxl,
                       "wet_cells": m.wet_cells, "diso": bool(m.cfg.diso), "precision": "fp64 plain",
                       "l2": "flushed before every timed step (state 3.5 MB < L2)", "parallelism": f"replicas{world}"},
            "e2e": {"value": e2e_value, "unit": "tracer cell-updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "note": "per step: forcing + u H2D (pinned), step, rho D2H; L2 not flushed"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "kernel": "k_step_fp64", "algorithmic_bytes_per_launch": alg,
                         "note": "plain FP64 form is FP64-issue bound on GB300, not HBM bound"},
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
