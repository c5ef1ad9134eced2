"""Benchmark: cell-updates/s of the ADER-WENO step on one GB300.

Default workload (--workload stiff): 2-D Euler + relaxing heat flux
(Cattaneo), 7 variables (rho, rho u, rho v, E, q_x, q_y, log10 tau),
1024x1024 periodic cells on [0,1]^2, order N=2, Rusanov, CFL 0.8, stiff
Newton predictor to ||obj||_inf <= 1e-12, tau piecewise constant on 16x16
patches with log10 tau ~ U(-7,-2) (pypde_gb300.workloads.relaxation, seeded
synthetic data).  Forms measured on the same K steps from the same state:
  plain          Newton from the plain guess q = w
  learned        Newton from the learned warm start (network trained here on
                 20 harvested plain steps with the library's own kernels;
                 training time reported, not timed in `value`), used only
                 if it needed fewer Newton iterations than the plain guess
                 on held-out harvested cells (else the plain guess stays)
  learned_network  the network's guess used regardless of that check
  mixed          FP32 Newton sweeps, then >= 2 FP64 sweeps to the same 1e-12
  learned_mixed  both
`value` is the learned form (the metric's "learned" form); `forms` gives
each with its Newton iterations and its relative L1 error per variable
against the CPU oracle (oracle/, the C restatement of the reference's step,
all host cores) run over the same K steps from the same initial state
(`l1_vs_oracle`; `oracle_check.plain_bit_identical` says whether the plain
form equals it bit for bit), and against the same steps converged to Newton
tolerance 1e-15 (`l1_vs_converged`: the 1e-12 tolerance's own effect).
--workload shear: 2-D Euler shear layer 512x512 N=3, plain FP64 (Picard).

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference]
                  [--workload stiff|shear]

Our arm prints one JSON line:
  value        cell-updates/s with the state resident in HBM, timed by CUDA
               events on the library's stream around exactly K steps
  e2e          the same metric through the public API (pypde_gb300.pde_solver)
               from a pinned host array: host->device copy of the state,
               K steps, device->host copy of the final state and the
               snapshot row, all inside the timed region
  roofline     the dominant kernel (the larger of the faces stage, k_faces or
               the Rusanov pair k_faces_pre + k_faces_eig, and the predictor,
               k_newton or k_predictor; FP64-bound): algorithmic
               FP64 flops of one launch (pypde_gb300.work_model) / its mean
               launch time measured here with CUDA events, against the FP64
               FMA peak measured here (MEASURED_PEAKS.json has no FP64
               figure); the other kernel's entry stands beside it
  cpu_baseline the CPU oracle's run of the K timed steps (the C restatement
               of the reference, oracle/, on all host cores; the 3-D
               workload on a stated 48^3 grid)
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
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "cell_updates_per_s"
UNIT = "cell-updates/s"

WORKLOADS = {
    # name: (system, ndim, n, N, cfl, stiff)
    "stiff": ("cattaneo", 2, 1024, 2, 0.8, True),
    "stiff3d": ("cattaneo", 3, 256, 2, 0.8, True),
    "shear": ("euler", 2, 512, 3, 0.8, False),
}

# DRAM bytes (read + write) of the faces stage per face point (the Rusanov
# pair k_faces_pre + k_faces_eig), from ncu captures of smaller grids of
# the same workload (a full-size stage is scaled by its face points): the
# relaxation system at 512^2, N=2 (k_faces_pre 0.241 GB read + 1.633 GB
# written, k_faces_eig 1.306 + 1.412 GB, over 2,101,248 face points).  Most
# of it is the records between the two kernels (73 doubles written and read
# per face point) and the eigen solver's stack lines evicted to DRAM.  The
# command lines are in the k_faces summaries under profiles/.
FACES_DRAM_BYTES_PER_POINT = {("cattaneo", 2, 2): 2185.4}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="stiff", choices=sorted(WORKLOADS))
    p.add_argument("--side", type=int, default=0, help="cells per side (0: the workload's)")
    p.add_argument("--order", type=int, default=0, help="N (0: the workload's)")
    p.add_argument("--train-iters", type=int, default=3000)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--batch-problems", type=int, default=256,
                   help="problems of the batched section (0: skip it)")
    p.add_argument("--batch-steps", type=int, default=6)
    p.add_argument("--batch-full", action="store_true",
                   help="batched section: every problem to its own tf (plain form only)")
    p.add_argument("--strips", type=int, default=0,
                   help="predictor strips overlapped with the faces (0: the library's choice, "
                        "1: none)")
    p.add_argument("--forms", default="all",
                   help="stiff workloads: comma list of forms to time besides the head "
                        "(plain,mixed,learned_mixed,learned_network) or 'all'")
    a = p.parse_args()
    system, ndim, n, N, cfl, stiff = WORKLOADS[a.workload]
    a.system, a.ndim, a.cfl, a.stiff = system, ndim, cfl, stiff
    a.n = a.side or n
    a.order = a.order or N
    return a


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


def l1(a, b):
    """Relative L1 error per variable: sum|a-b| / sum|b| over all cells."""
    ax = tuple(range(a.ndim - 1))
    return np.abs(a - b).sum(axis=ax) / np.abs(b).sum(axis=ax)


def initial_state(args, seed):
    from pypde_gb300 import workloads
    if args.workload == "stiff":
        return workloads.relaxation(args.n, 2, seed=seed)
    if args.workload == "stiff3d":
        return workloads.relaxation(args.n, 3, seed=seed, log10_tau=(-6.0, -3.0), amp=0.05)
    return workloads.shear(args.n, seed=seed)


def workload_name(args):
    if args.workload == "stiff3d":
        return (f"3-D Euler + relaxing heat flux (9 vars), {args.n}^3 periodic, N={args.order}, "
                f"Rusanov, CFL {args.cfl}, stiff Newton predictor to 1e-12, log10 tau ~ "
                "U(-6,-3) per octant")
    if args.workload == "stiff":
        return (f"2-D Euler + relaxing heat flux (7 vars), {args.n}x{args.n} periodic, "
                f"N={args.order}, Rusanov, CFL {args.cfl}, stiff Newton predictor to 1e-12, "
                "log10 tau ~ U(-7,-2) on 16x16 patches")
    return (f"2-D Euler shear layer {args.n}x{args.n} periodic, N={args.order}, Rusanov, "
            f"CFL {args.cfl}, plain FP64 (Picard predictor)")


def cpu_run(args, u, steps, cores):
    from oracle import ora
    return ora.pde_solver(args.system, u, 10.0, [1.0] * args.ndim, [1] * args.ndim, args.cfl,
                          args.order,
                          stiff=args.stiff, max_steps=steps, nthreads=cores)


def oracle_check(args, u0, local, warm, forms):
    """The CPU oracle (all host cores) for the timed region's K steps from
    the initial state, on the workload's own grid (the 3-D workload on a
    48^3 grid of the same kind: its full grid takes the host minutes per
    step); each GPU form runs the same steps on the same grid.  Returns
    the per-form relative L1 per variable ("l1"), whether the plain form
    is bit-identical to the oracle, and the oracle's run as the CPU
    baseline."""
    import copy
    cores = os.cpu_count() or 1
    a = args
    if args.ndim == 3 and args.n > 48:
        from pypde_gb300 import workloads
        a = copy.copy(args)
        a.n = 48
        u0 = workloads.relaxation(48, 3, seed=0, log10_tau=(-6.0, -3.0), amp=0.05)
    C = int(np.prod(u0.shape[:-1]))
    t0 = time.perf_counter()
    u_o, _, k, _ = cpu_run(a, u0, args.steps, cores)
    el = time.perf_counter() - t0
    R = Runner(a, local)
    l1s, bitwise = {}, None
    for name, w, mx, force in forms:
        q = u0.copy()
        R.run(q, args.steps, warm=w, mixed=mx, force=force)
        l1s[name] = [float(x) for x in l1(q, u_o)]
        if name == "plain":
            bitwise = bool(np.array_equal(q, u_o))
    grid = "x".join(map(str, u0.shape[:-1]))
    return {"l1": l1s, "grid": grid, "steps": k, "plain_bit_identical": bitwise,
            "oracle": "the C restatement of the reference's step (oracle/ader_oracle.c), "
                      "Newton tolerance 1e-12 for the stiff forms",
            "cpu_baseline": {"value": C * k / el, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"the oracle's {k} whole-grid steps on a {grid} grid, "
                                       f"N={args.order}, from the initial state, {el:.1f} s"}}


class Runner:
    """Timed runs of the solver through the C ABI (pde_solver_ex)."""

    def __init__(self, args, local):
        from pypde_gb300 import _lib
        from pypde_gb300.callbacks import builtin_system
        self.L = _lib.lib()
        self._lib = _lib
        self.args, self.local = args, local
        self.sys = builtin_system(args.system, args.ndim)
        self.nX = np.array([args.n] * args.ndim, dtype=np.int32)
        self.dX = np.array([1.0 / args.n] * args.ndim)
        self.bt = np.array([1] * args.ndim, dtype=np.int32)

    def run(self, u, steps, profile=False, warm=None, tol=0.0, mixed=False, force=False,
            tf=10.0):
        """warm: a WarmStart, used as pde_solver uses it (only if its
        validation found a saving), or always with force.  steps < 0: run
        to tf."""
        _lib, a = self._lib, self.args
        if warm is not None and not (force or warm.active):
            warm = None
        opt = _lib.Options()
        opt.mixed_precision = int(mixed)
        opt.max_steps = steps
        opt.device = self.local
        opt.profile_stages = int(profile)
        opt.newton_tol = tol
        opt.strips = a.strips
        if warm is not None:
            opt.warm_start = warm.handle
        st = _lib.Stats()
        s = self.sys
        _lib.check(self.L.pde_solver_ex(s.handle, s.has_F, s.has_B, s.has_S, _lib.c_ptr(u),
                                        float(tf), _lib.c_ptr(self.nX), a.ndim,
                                        _lib.c_ptr(self.dX),
                                        a.cfl, _lib.c_ptr(self.bt), a.stiff, 0, a.order, 1,
                                        None, opt, st))
        return st.as_dict()


def measure_form(R, args, ws, u0, warm=None, mixed=False, force=False):
    """W warm-up steps, then exactly K timed steps (CUDA events inside the
    library), then an eagerly launched profile of min(K, 5) steps from the
    same state as the timed steps."""
    u = u0.copy()
    R.run(u, args.warmup, warm=warm, mixed=mixed, force=force)
    u_warm = u.copy()
    barrier(ws)
    st = R.run(u, args.steps, warm=warm, mixed=mixed, force=force)
    barrier(ws)
    sec = allmax(ws, st["device_seconds"])
    ksteps = max(1, min(args.steps, 5))
    sp = R.run(u_warm.copy(), ksteps, profile=True, warm=warm, mixed=mixed, force=force)
    return st, sec, sp, ksteps, u_warm


def run_batched(args, local):
    """Uneven batch (256 problems, side log-uniform in [64, 512], order in
    {1, 2, 3}, 2-D Euler + relaxation, stiff Newton): one pde_solver_batch
    call against the same problems solved one after the other, both for
    the same number of steps per problem (the autotuner's 4 timed steps
    included in the batched time)."""
    from pypde_gb300 import systems, workloads
    from pypde_gb300.solvers import pde_solver, pde_solver_batch
    s = systems.cattaneo(2)
    K = args.batch_steps
    probs = workloads.batched(args.batch_problems, seed=0)
    for N in (1, 2, 3):  # load the kernels before timing
        q = np.ascontiguousarray(workloads.relaxation(16, 2))
        pde_solver(q, 1.0, [1, 1], F=s.F, S=s.S, boundaryTypes="periodic", order=N,
                   stiff=True, max_steps=2, device=local)
    b = [dict(p, Q0=p["Q0"].copy()) for p in probs]
    st = {}
    pde_solver_batch(b, F=s.F, S=s.S, stiff=True, max_steps=None if args.batch_full else K,
                     stats=st, device=local)
    upd = sum(p["Q0"].shape[0] * p["Q0"].shape[1] * k
              for p, k in zip(probs, st["steps_per_problem"]))
    if args.batch_full:  # every problem to its own tf, the batched launch alone
        return {"problems": len(probs), "to_tf": float(probs[0]["tf"]),
                "cells": int(sum(p["Q0"].shape[0] * p["Q0"].shape[1] for p in probs)),
                "steps_per_problem_min_max": [int(min(st["steps_per_problem"])),
                                              int(max(st["steps_per_problem"]))],
                "cell_updates": int(upd),
                "batched": {"value": upd / st["device_seconds"], "unit": UNIT,
                            "seconds": st["device_seconds"], "tune_seconds": st["tune_seconds"],
                            "newton_iters": st["pred_iters"], "nan_found": st["nan_found"]}}
    seq = 0.0
    same = True
    for p, pb in zip(probs, b):
        q = p["Q0"].copy()
        s1 = {}
        pde_solver(q, p["tf"], p["L"], F=s.F, S=s.S, boundaryTypes="periodic", cfl=p["cfl"],
                   order=p["order"], stiff=True, max_steps=K, stats=s1, device=local)
        seq += s1["device_seconds"]
        same &= bool(np.array_equal(q, pb["Q0"]))
    # the learned form through the batch: one network per order, trained on
    # a 64^2 problem of that order and validated like the one-problem form
    # (gated); its own guess forced on; and the FP32-sweep form.  Each
    # against the plain batched result (relative L1, largest over problems)
    from pypde_gb300 import warmstart
    nets, gates = {}, {}
    for N in (1, 2, 3):
        u0 = workloads.relaxation(64, 2, seed=40 + N, patches=4)
        ws = warmstart.train_warm_start(u0, 10.0, [1.0, 1.0], F=s.F, S=s.S, cfl=0.8, order=N,
                                        tau_var=6, steps=8, per_step=1024, iters=300, seed=N,
                                        device=local)
        nets[N], gates[N] = ws, {"active": bool(ws.active), **ws.validation}

    def batched_form(**opts):
        bb = [dict(p, Q0=p["Q0"].copy()) for p in probs]
        st2 = {}
        pde_solver_batch(bb, F=s.F, S=s.S, stiff=True, max_steps=K, stats=st2, device=local,
                         **opts)
        err = max(float(l1(q2["Q0"], q1["Q0"]).max()) for q2, q1 in zip(bb, b))
        return {"value": upd / st2["device_seconds"], "unit": UNIT,
                "seconds": st2["device_seconds"],
                "over_sequential_plain": seq / st2["device_seconds"],
                "newton_iters": st2["pred_iters"], "l1_vs_plain_batched": err}

    forms = {"learned": batched_form(warm_start=nets)}
    for ws in nets.values():
        ws.active = True
    forms["learned_network"] = batched_form(warm_start=nets)
    forms["mixed"] = batched_form(mixed_precision=True)
    forms["plain_newton_iters"] = st["pred_iters"]
    forms["warm_start_gates"] = gates
    orders = np.bincount([p["order"] for p in probs], minlength=4)[1:].tolist()
    return {"problems": len(probs), "orders_1_2_3": orders,
            "cells": int(sum(p["Q0"].shape[0] * p["Q0"].shape[1] for p in probs)),
            "steps_per_problem": K, "cell_updates": int(upd),
            "batched": {"value": upd / st["device_seconds"], "unit": UNIT,
                        "seconds": st["device_seconds"], "tune_seconds": st["tune_seconds"],
                        "kernel_launches": st["kernel_launches"],
                        "tiles_per_pop": st["per_pop"]},
            "sequential": {"value": upd / seq, "unit": UNIT, "seconds": seq},
            "batched_over_sequential": seq / st["device_seconds"],
            "bit_identical_to_sequential": same,
            "forms": forms}


def run_ours(args, ws, rank, local):
    from pypde_gb300 import _lib, systems, work_model
    from pypde_gb300.solvers import pde_solver

    L = _lib.lib()
    n, N, nd = args.n, args.order, args.ndim
    V = 2 * nd + 3 if args.system == "cattaneo" else nd + 2
    C = n ** nd
    Cw = (n + 2) ** nd
    Ls = [1.0] * nd
    u0 = initial_state(args, rank)
    R = Runner(args, local)
    peak = _lib.ctypes.c_double()
    _lib.check(L.pypde_measure_fp64_peak(local, peak))
    dmma = _lib.ctypes.c_double()
    _lib.check(L.pypde_measure_dmma_peak(local, dmma))
    s = systems.cattaneo(nd) if args.system == "cattaneo" else systems.euler(nd)

    forms = {}
    warm = None
    train = None
    # the stiff workloads' forms: all five, or (--forms) plain and the ones
    # listed, without the network when no learned form is listed
    allf = ["plain", "mixed", "learned_mixed", "learned_network"]
    sel = allf if args.forms == "all" else [f for f in args.forms.split(",") if f in allf]
    learned = args.stiff and (args.forms == "all" or any("learned" in f for f in sel))
    if learned:
        from pypde_gb300 import warmstart
        t0 = time.perf_counter()
        warm = warmstart.train_warm_start(u0, 10.0, Ls, F=s.F, S=s.S, cfl=args.cfl,
                                          order=N, tau_var=2 * nd + 2, steps=20, per_step=16384,
                                          iters=args.train_iters, seed=rank, device=local)
        train = {"seconds": time.perf_counter() - t0, "samples": warm.samples,
                 "iters": args.train_iters, "train_rms_normalised": warm.train_rms,
                 "harvest": "20 plain steps from the initial state, 16384 cells per step; "
                            "the last step's sample held out for validation",
                 "validation": warm.validation, "active": bool(warm.active),
                 "gate": "the learned form uses the network only if it needed fewer Newton "
                         "iterations than the plain guess on the held-out cells; otherwise "
                         "it keeps the plain guess (form learned_network forces it)"}

    head = "learned" if learned else "plain"
    with Clocks(local) as clk:
        st_h, sec, sp, ksteps, u_warm = measure_form(R, args, ws, u0, warm)
    forms[head] = (st_h, sec, sp, ksteps)
    # (name, warm start, FP32 sweeps, network forced)
    spec = {"plain": (None, False, False), "learned": (warm, False, False),
            "mixed": (None, True, False), "learned_mixed": (warm, True, False),
            "learned_network": (warm, False, True)}
    if args.stiff:
        for f in sel:
            if f not in forms:
                w, mx, fc = spec[f]
                forms[f] = measure_form(R, args, ws, u0, w, mixed=mx, force=fc)[:4]
    value = ws * C * args.steps / sec

    # every form against the CPU oracle over the same K steps from u0, and
    # against the same steps converged to Newton tolerance 1e-15 (the
    # 1e-12 tolerance's own effect)
    errs, conv_errs, oracle = {}, {}, None
    if rank == 0 and ws == 1 and not args.no_cpu:
        oracle = oracle_check(args, u0, local, warm, [(f,) + spec[f] for f in forms])
        errs = oracle.pop("l1")
    if args.stiff:
        q_o = u0.copy()
        R.run(q_o, args.steps, tol=1e-15)
        for name in forms:
            w, mx, force = spec[name]
            q = u0.copy()
            R.run(q, args.steps, warm=w, mixed=mx, force=force)
            conv_errs[name] = [float(x) for x in l1(q, q_o)]

    def form_summary(name):
        st, sec_f, sp_f, ks = forms[name]
        its = st["pred_iters"] / (args.steps * Cw)
        d = {"value": ws * C * args.steps / sec_f, "ms_per_step": 1e3 * sec_f / args.steps,
             "predictor_iters_per_cell": its,
             "stage_ms_per_step": {k: 1e3 * v / ks for k, v in sp_f["stage_seconds"].items()}}
        if args.stiff:
            d["newton_fallbacks"] = st["pred_fallbacks"]
            d["fp32_sweeps_per_cell"] = st["pred_iters32"] / (args.steps * Cw)
            d["l1_vs_converged"] = conv_errs[name]
        if name in errs:
            d["l1_vs_oracle"] = errs[name]
        return d

    full = None
    if args.workload == "shear":
        # the shear layer's whole run to its end time tf = 0.5 (CFL 0.8)
        q = u0.copy()
        stf = R.run(q, -1, tf=0.5)
        full = {"tf": 0.5, "steps": stf["steps"], "seconds": stf["device_seconds"],
                "value": ws * C * stf["steps"] / stf["device_seconds"], "unit": UNIT,
                "t_final": stf["t_final"], "nan_found": bool(stf["nan_found"])}
    stage_s = sp["stage_seconds"]
    its = sp["pred_iters"] / (ksteps * Cw)
    fpf = work_model.face_point_flops(args.system, nd, V, N)
    fpts = work_model.face_points([n] * nd, N)
    faces_launch = stage_s["faces"] / ksteps
    achieved = fpts * fpf / faces_launch / 1e12
    # the predictor kernel: its useful work is the iterations the plain
    # form needs from the same state (a warm start that saves iterations
    # shows as a higher rate), over its mean launch time in the timed form
    sp_plain = forms["plain"][2] if "plain" in forms else sp
    ks_plain = forms["plain"][3] if "plain" in forms else ksteps
    its_plain = sp_plain["pred_iters"] / (ks_plain * Cw)
    per_it = (work_model.newton_flops_per_iteration if args.stiff
              else work_model.predictor_flops_per_iteration)(args.system, nd, V, N)
    pred_launch = stage_s["predictor"] / ksteps
    pred_flops = Cw * its_plain * per_it
    pred_kernel = "k_newton" if args.stiff else "k_predictor"
    roof_pred = {"bound": "fp64", "kernel": pred_kernel,
                 "achieved": pred_flops / pred_launch / 1e12, "peak": peak.value,
                 "unit": "TFLOP/s", "frac": pred_flops / pred_launch / 1e12 / peak.value,
                 "traffic": None, "traffic_source": "none: no ncu capture of this kernel "
                                                     "at this size",
                 "peak_source": "FP64 FMA loop measured by this run "
                                "(MEASURED_PEAKS.json has no FP64 figure)",
                 "flops_per_launch": pred_flops, "launch_ms": 1e3 * pred_launch,
                 "iters_per_cell_counted": its_plain, "iters_per_cell_run": its,
                 "note": "algorithmic flops of " + ("the Newton iteration (residual, FD "
                         "Jacobian of S, dense LU and solve of each spatial node's (N V)^2 "
                         "system)" if args.stiff else "the Picard iteration") +
                         " per w-cell, times the iterations the plain form takes from the "
                         "same state (pypde_gb300.work_model); the launch time includes "
                         "the warm-start network's guess kernel in the learned form"}
    per_point = FACES_DRAM_BYTES_PER_POINT.get((args.system, nd, N))
    traffic = None if per_point is None else per_point * fpts
    traffic_src = ("none: no ncu capture of this workload" if per_point is None else
                   f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_faces_pre + "
                   f"k_faces_eig pair of this workload captured on another grid size, "
                   f"{per_point:.0f} B per face point, "
                   f"times {fpts} face points; the algorithmic bytes are "
                   f"{work_model.faces_bytes_per_launch([n] * nd, V, N):.3e}")
    flops = work_model.step_flops(args.system, [n] * nd, V, N, its, stiff=args.stiff)

    # e2e through the public API from pinned host memory (the headline form),
    # over the same K steps as the timed region (from the warmed-up state)
    try:
        import torch
        pinned = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        pinned = np.empty(u0.shape)
    pinned[...] = u_warm
    barrier(ws)
    t0 = time.perf_counter()
    pde_solver(pinned, 10.0, Ls, F=s.F, S=s.S if args.stiff else None,
               boundaryTypes="periodic", cfl=args.cfl, order=N, ndt=1, stiff=args.stiff,
               max_steps=args.steps, device=local, warm_start=warm if args.stiff else None,
               strips=args.strips)
    e2e_s = allmax(ws, time.perf_counter() - t0)
    barrier(ws)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args), "form": head, "cells": C, "order": N,
                   "vars": V, "strips": args.strips or "library's choice",
                   "l2": "working set > L2 (qh alone is "
                         f"{Cw * N ** (nd + 1) * V * 8 / 1e6:.0f} MB); no flush",
                   "parallelism": f"replicas x{ws}"},
        "forms": {k: form_summary(k) for k in forms},
        "e2e": {"value": ws * C * args.steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": C * V * 8 / args.steps,
                "d2h_bytes_per_step": 2 * C * V * 8 / args.steps,
                "note": "one pde_solver call advancing the same K steps as the timed "
                        "region (from the state after the warm-up): the state goes in "
                        "once, the final state plus the snapshot row come out once"},
        "roofline": None,
        "roofline_faces": {"bound": "fp64", "kernel": "k_faces_pre + k_faces_eig (Rusanov "
                           "faces in two launches)", "achieved": achieved,
                     "peak": peak.value, "unit": "TFLOP/s", "frac": achieved / peak.value,
                     "traffic": traffic,
                     "traffic_source": traffic_src,
                     "peak_source": "FP64 FMA loop measured by this run "
                                    "(MEASURED_PEAKS.json has no FP64 figure)",
                     "flops_per_launch": fpts * fpf, "launch_ms": 1e3 * faces_launch,
                     "note": "algorithmic flops count max|eig| as the nominal 10 m^3 of a "
                             "Hessenberg + Francis QR of the m x m active block of the flux "
                             "Jacobian (m = V, or V minus the system's passive variables); "
                             "the kernel's mixed-precision eigensolver does less FP64 work "
                             "than that; launch_ms is the faces stage timed alone (both "
                             "kernels); the records between the two kernels add 1168 B of "
                             "DRAM traffic per face point to a stage that is FP64-bound "
                             "(DRAM under 10% of its peak)"},
        "stage_ms_per_step": {k: 1e3 * v / ksteps for k, v in stage_s.items()},
        "step_fp64_tflops": sum(flops.values()) / (sec / args.steps) / 1e12,
        "fp64_pipes": {"fma_tflops": peak.value, "dmma_tflops": dmma.value,
                       "note": "FP64 FMA loop and FP64 tensor-core mma.sync m8n8k4 loop, both "
                               "measured by this run: the predictor's contractions could "
                               "gain from DMMA only if the second were above the first"},
        "predictor_iters_per_cell": its,
        "gpu_launches": st_h["kernel_launches"],
        "clocks": clk.summary(),
    }
    # the dominant kernel's roofline is the headline one, the other beside it
    if pred_launch >= faces_launch:
        out["roofline"], out["roofline_predictor"] = roof_pred, None
        del out["roofline_predictor"]
    else:
        out["roofline"] = out.pop("roofline_faces")
        out["roofline_predictor"] = roof_pred
    if train:
        out["training"] = train
    if full:
        out["full_run"] = full
    if args.stiff and args.batch_problems > 0 and ws == 1:
        out["batched_workload"] = run_batched(args, local)
    if oracle is not None:
        out["cpu_baseline"] = oracle.pop("cpu_baseline")
        out["oracle_check"] = oracle
    return out


def run_reference(args, ws, rank):
    """The reference's algorithm on the host cores (the C restatement; the
    reference's own build needs its source tree, absent on the GPU host)."""
    if rank != 0:
        return None
    u = initial_state(args, 0)
    cores = os.cpu_count() or 1
    n = args.n
    cpu_run(args, u, args.warmup, cores)
    t0 = time.perf_counter()
    u, _, k, _ = cpu_run(args, u, args.steps, cores)
    el = time.perf_counter() - t0
    v = n ** args.ndim * k / el
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / k,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": workload_name(args), "form": "plain",
                       "cells": n ** args.ndim},
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
