"""Benchmark: cell-updates/s of the ADER-WENO step on one GB300.

Workload (default): 2-D Euler shear layer, 512x512 periodic cells on [0,1]^2,
order N=3, Rusanov flux, CFL 0.8, plain FP64 form (the Picard predictor) --
the configuration the reference's plain GPU-vs-CPU comparison is quoted on.
Seeded synthetic initial state (pypde_gb300.workloads.shear).  One step is
one ADER time step over the whole grid.

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference]

Our arm prints one JSON line:
  value        cell-updates/s with the state resident in HBM, timed by CUDA
               events on the library's stream around exactly K steps
  e2e          the same metric through the public API (pypde_gb300.pde_solver)
               from a pinned host array: host->device copy of the state,
               K steps, device->host copy of the final state and the
               snapshot row, all inside the timed region
  roofline     the dominant kernel (k_faces, FP64-bound): algorithmic FP64
               flops of one launch (pypde_gb300.work_model) / its mean launch
               time measured here with CUDA events, against the FP64 FMA
               peak measured here (MEASURED_PEAKS.json has no FP64 figure)
  cpu_baseline the CPU restatement of the reference (oracle/) on all host
               cores, on a bounded sample (stated)
The reference arm (--impl reference) times that CPU path alone.

Multi-GPU: the reference's only parallelism is an x-slab split of one grid;
this bench runs replicas (one independent grid per GPU, no exchange) under
torchrun, barrier + max over ranks, and reports the aggregate ("weak").
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "cell_updates_per_s"
UNIT = "cell-updates/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=512, help="cells per side")
    p.add_argument("--order", type=int, default=3)
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="budget of the CPU-baseline sample")
    p.add_argument("--no-cpu", action="store_true")
    return p.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region (200 ms)."""

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.device}",
                                       f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
        self.f.flush()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines()]
        except OSError:
            rows = []
        os.unlink(self.f.name)
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit()
                else None, "reasons": sorted(reasons), "samples": len(rows)}


def cpu_baseline(u0, N, cfl, budget):
    """The CPU restatement on all host cores: whole-grid steps until the
    budget is used (at least one step).  Returns (cell-updates/s, cores,
    sample description)."""
    from oracle import ora
    cores = os.cpu_count() or 1
    C = int(np.prod(u0.shape[:-1]))
    u = u0
    steps, t0 = 0, time.perf_counter()
    while True:
        u, _, k, _ = ora.pde_solver("euler", u, 10.0, [1.0, 1.0], [1, 1], cfl, N, max_steps=1,
                                    nthreads=cores)
        steps += k
        el = time.perf_counter() - t0
        if el >= budget or steps >= 50:
            break
    sample = (f"{steps} whole-grid step(s) of the same {u0.shape[0]}x{u0.shape[1]} N={N} "
              f"workload, {el:.1f} s")
    return C * steps / el, cores, sample


def run_ours(args, ws, rank, local):
    from pypde_gb300 import _lib, systems, work_model, workloads
    from pypde_gb300.callbacks import builtin_system
    from pypde_gb300.solvers import pde_solver

    L = _lib.lib()
    n, N, cfl, V = args.n, args.order, 0.8, 4
    C = n * n
    u0 = workloads.shear(n, seed=rank)
    sysobj = builtin_system("euler", 2)
    nX = np.array([n, n], dtype=np.int32)
    dX = np.array([1.0 / n, 1.0 / n])
    bt = np.array([1, 1], dtype=np.int32)

    def run(u, steps, profile=False):
        opt = _lib.Options()
        opt.max_steps = steps
        opt.device = local
        opt.profile_stages = int(profile)
        st = _lib.Stats()
        _lib.check(L.pde_solver_ex(sysobj.handle, True, False, False, _lib.c_ptr(u), 10.0,
                                   _lib.c_ptr(nX), 2, _lib.c_ptr(dX), cfl, _lib.c_ptr(bt),
                                   False, 0, N, 1, None, opt, st))
        return st

    # warm-up: W steps (module load, arena allocation, graph capture)
    u = u0.copy()
    run(u, args.warmup)
    peak = _lib.ctypes.c_double()
    _lib.check(L.pypde_measure_fp64_peak(local, peak))

    # timed: exactly K steps, state resident in HBM, CUDA events inside
    barrier(ws)
    with Clocks(local) as clk:
        st = run(u, args.steps)
    barrier(ws)
    sec = allmax(ws, st.device_seconds)
    value = ws * C * args.steps / sec

    # stage profile of the same workload (eager launches, events per stage)
    ksteps = max(1, min(args.steps, 5))
    sp = run(u0.copy(), ksteps, profile=True).as_dict()
    stage_s = sp["stage_seconds"]
    its = sp["pred_iters"] / (ksteps * (n + 2) ** 2)
    fpf = work_model.face_point_flops("euler", 2, V, N)
    fpts = work_model.face_points([n, n], N)
    faces_launch = stage_s["faces"] / ksteps
    achieved = fpts * fpf / faces_launch / 1e12
    flops = work_model.step_flops("euler", [n, n], V, N, its)

    # e2e through the public API from pinned host memory
    try:
        import torch
        pinned = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        pinned = np.empty(u0.shape)
    pinned[...] = u0
    s = systems.euler(2)
    barrier(ws)
    t0 = time.perf_counter()
    pde_solver(pinned, 10.0, [1.0, 1.0], F=s.F, boundaryTypes="periodic", cfl=cfl, order=N,
               ndt=1, stiff=False, max_steps=args.steps, device=local)
    e2e_s = allmax(ws, time.perf_counter() - t0)
    barrier(ws)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"2-D Euler shear layer {n}x{n} periodic, N={N}, Rusanov, "
                               f"CFL {cfl}, plain FP64 (Picard predictor)",
                   "cells": C, "order": N, "vars": V,
                   "l2": "working set > L2 (qh alone is "
                         f"{(n + 2) ** 2 * N ** 3 * V * 8 / 1e6:.0f} MB); no flush",
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": ws * C * args.steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": C * V * 8 / args.steps,
                "d2h_bytes_per_step": 2 * C * V * 8 / args.steps,
                "note": "one pde_solver call advancing K steps: the state goes in once and "
                        "the final state plus the snapshot row come out once"},
        "roofline": {"bound": "fp64", "kernel": "k_faces", "achieved": achieved,
                     "peak": peak.value, "unit": "TFLOP/s", "frac": achieved / peak.value,
                     "traffic": None,
                     "peak_source": "FP64 FMA loop measured by this run "
                                    "(MEASURED_PEAKS.json has no FP64 figure)",
                     "flops_per_launch": fpts * fpf, "launch_ms": 1e3 * faces_launch},
        "stage_ms_per_step": {k: 1e3 * v / ksteps for k, v in stage_s.items()},
        "step_fp64_tflops": sum(flops.values()) / (sec / args.steps) / 1e12,
        "predictor_iters_per_cell": its,
        "gpu_launches": st.kernel_launches,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu:
        v, cores, sample = cpu_baseline(u0, N, cfl, args.cpu_seconds)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": sample}
    return out


def run_reference(args, ws, rank):
    """The reference's algorithm on the host cores (the C restatement; the
    reference's own build needs its source tree, absent on the GPU host)."""
    if rank != 0:
        return None
    from pypde_gb300 import workloads
    n, N, cfl = args.n, args.order, 0.8
    u = workloads.shear(n)
    cores = os.cpu_count() or 1
    from oracle import ora
    ora.pde_solver("euler", u, 10.0, [1.0, 1.0], [1, 1], cfl, N, max_steps=args.warmup,
                   nthreads=cores)
    t0 = time.perf_counter()
    u, _, k, _ = ora.pde_solver("euler", u, 10.0, [1.0, 1.0], [1, 1], cfl, N,
                                max_steps=args.steps, nthreads=cores)
    el = time.perf_counter() - t0
    v = n * n * k / el
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / k,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"2-D Euler shear layer {n}x{n} periodic, N={N}, "
                                   f"Rusanov, CFL {cfl}, plain FP64", "cells": n * n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{k} whole-grid steps after {args.warmup} warm-up"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        out = run_reference(args, ws, rank)
    else:
        out = run_ours(args, ws, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
