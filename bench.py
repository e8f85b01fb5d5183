#!/usr/bin/env python
"""Implicit-step throughput of the phi + c CALPHAD level on GB300.

Workload (default): one uniform periodic 256^3 level, phi + binary c, CALPHAD
regular solution with two Redlich-Kister coefficients per phase, T_run plus a
50 K gradient along x, simple 7-point phase flux, EBS composition flux; BDF
Newton-GMRES(5) steps of dt = 0.1 with the multigrid-preconditioned FAC
blocks.  A "step" is one accepted implicit step of the whole level.

metric: implicit-step cell-updates/s = cells x accepted steps / time.
  value : device time (CUDA events on the stepper's stream), state resident.
  e2e   : wall time through the public C-ABI with the state handed in from
          pinned host memory and read back every step.
Runs on N GPUs as N independent replicas (the level is not sharded).

--impl reference: the CPU restatement of the reference path (the oracle in
oracle/, all host threads) on a bounded sample of the same workload.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "implicit-step cell-updates/s, mixed+surrogate vs plain FP64, at ≤1e-6 rel L2 err"
UNIT = "cell-updates/s"
# algorithmic bytes per cell and launch of the per-cell KKS Newton kernel:
# read phi, c, cL_ref, cS_ref (4 x 8 B), write cL, cS, dF (3 x 8 B)
KKS_BYTES_PER_CELL = 56
RHS_BYTES_PER_CELL = 56  # read phi, phi_lag, cL, cS, dF; write phi', c'
# mixed path KKS kernel: read phi, c (FP64), cL_ref, cS_ref (FP32); write cL,
# cS, dF (FP32)
KKS_MIXED_BYTES_PER_CELL = 36
# mixed RHS evaluation, three launches: FP32 copy of phi (read 8, write 4),
# composition face weights (read phi 4, write 2 weights x 3 faces 24), RHS
# (read phi FP64 8, phi FP32 4, cL, cS 8, dF 4, face weights 24; write phi',
# c' FP64 16)
RHS_MIXED_BYTES_PER_CELL = 12 + 28 + 64
# analytic Jv on FP32 Krylov vectors: point pass 32 B (v 8, phi 4, cL, cS 8;
# write dphi, dcL, dcS 12) + stencil pass 68 B (dphi, dcL, dcS 12, face
# weights 24, phi 4, cL, cS 8, dF 4, v 8; write out 8)
JV_BYTES_PER_CELL = 32 + 68
# one red-black sweep (two colour launches) on the finest multigrid level,
# FP32, per cell: phase block u r/w 8 + f 4 + C 4 = 16 B, composition block
# u r/w 8 + f 4 + D (3 faces in 3D, 2 in 2D) 12 / 8 B; the two blocks
# alternate: 20 B in 3D, 18 B in 2D (twice that in FP64)
SMOOTH_BYTES_PER_CELL = {3: 20, 2: 18}
SMOOTH_BYTES_PER_CELL_FP64 = {3: 40, 2: 36}
# DRAM bytes per cell of one finest-level sweep of the FP32 smoother on the
# 3D CALPHAD phi + c level, from ncu (dram__bytes_read.sum +
# dram__bytes_write.sum) of the z-marching sweep's four launch kinds (phase
# and composition blocks, from zero and with the fused prolongation) at
# 224^3, averaged: 205.8 MB per launch over 11,239,424 cells
SMOOTH_DRAM_BYTES_PER_CELL_MEASURED = 18.3
# MLP inference: 2 (3*64 + 64*64 + 64*64 + 64*2) multiply-adds per cell
MLP_FLOPS_PER_CELL = 2 * (3 * 64 + 64 * 64 + 64 * 64 + 64 * 2)
KERNEL_NAMES = {
    False: {"kks_newton": "k_kks_f32+k_kks_polish64", "rhs_fused": "k_rhs_mixed",
            "jv_analytic": "k_jv_point+k_jv_stencil",
            "smooth_fine": {3: "k_sweep_z<float> (finest-level red-black sweep, one z-marching "
                               "launch)",
                            2: "k_rbgs_color<float,2> x2 (finest-level red-black sweep)"}},
    True: {"kks_newton": "k_kks_interior", "rhs_fused": "k_rhs_fused<0>",
           "jv_analytic": "-",
           "smooth_fine": {3: "k_sweep_z<double> (finest-level red-black sweep, one z-marching "
                              "launch)",
                           2: "k_rbgs_color<double,2> x2 (finest-level red-black sweep)"}},
}
# profiling-timer kinds of the stepper (ampe_stepper_kernel_time)
KINDS = ((0, "kks_newton"), (1, "rhs_fused"), (2, "jv_analytic"), (3, "mlp_infer_tc"),
         (4, "quat_rhs"), (5, "precond_solve"), (6, "precond_setup"), (7, "smooth_fine"))
SINGLE_KERNELS = ("kks_newton", "rhs_fused", "jv_analytic", "mlp_infer_tc", "smooth_fine")
ATOL = 1.0e-6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="calphad", choices=["calphad", "poly", "dendrite", "dilute"])
    ap.add_argument("--n", type=int, default=0, help="cells per side (0: the workload's)")
    ap.add_argument("--path", default="mixed+surrogate",
                    choices=["fp64", "mixed", "mixed+surrogate"])
    ap.add_argument("--surrogate-samples", type=int, default=1 << 22)
    ap.add_argument("--surrogate-steps", type=int, default=2000)
    ap.add_argument("--precond", type=int, default=2)
    ap.add_argument("--ref-atol", type=float, default=0.0,
                    help="also run the FP64 path at this tighter tolerance (untimed) and "
                         "report every path's error against it")
    ap.add_argument("--atol", type=float, default=ATOL,
                    help="Newton/WRMS absolute tolerance (rtol = atol/100)")
    ap.add_argument("--cpu-n", type=int, default=80,
                    help="side of the CPU sample level (3D: cpu_n^3, past the host caches)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--only-head", action="store_true",
                    help="time only the headline path (no FP64 / mixed comparison)")
    ap.add_argument("--surrogate-study-steps", type=int, default=200,
                    help="steps of the surrogate study (0: skip): from the cold initial state, "
                         "the plain warm start against the network's guess on cold starts "
                         "and for every KKS solve")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the headline path's timed steps with cudaProfilerStart/"
                         "Stop (ncu --profile-from-start off captures only them)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate(local_ms, local_cell_updates, group=None):
    """Max time over ranks and summed work (replicas): returns (ms, updates)."""
    import torch
    import torch.distributed as dist

    if group is None and not (dist.is_available() and dist.is_initialized()):
        return local_ms, local_cell_updates
    t = torch.tensor([local_ms], dtype=torch.float64)
    w = torch.tensor([float(local_cell_updates)], dtype=torch.float64)
    backend = dist.get_backend(group)
    if backend == "nccl":
        t, w = t.cuda(), w.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(w, op=dist.ReduceOp.SUM, group=group)
    return float(t.item()), float(w.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            time.sleep(0.3)  # let the sampler start before the timed region
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.th.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def kernel_rooflines(kt, per_cell, N, pk):
    """Achieved algorithmic bandwidth (GB/s) or tensor rate (TFLOP/s) of every
    instrumented kernel kind: bytes (or FLOP) per cell x cells x launches over
    the kind's summed CUDA-event time."""
    out = {}
    for k, v in kt.items():
        if not v["launches"] or v["ms"] <= 0.0:
            continue
        sec = v["ms"] / 1e3
        if k == "mlp_infer_tc":
            a = MLP_FLOPS_PER_CELL * N * v["launches"] / sec / 1e12
            out[k] = {"achieved": a, "unit": "TFLOP/s", "frac": a / pk["bf16_tflops"]}
        elif k in per_cell:
            a = per_cell[k] * N * v["launches"] / sec / 1e9
            out[k] = {"achieved": a, "unit": "GB/s", "frac": a / pk["hbm_gbs"],
                      "bytes_per_cell": per_cell[k]}
    return out


def kks_issue(roofs, kt, res):
    """The per-cell KKS Newton is bound by instruction issue (FP32 FMA and
    MUFU logarithms per iteration), not by its bytes: its rate is Newton
    iterations per second; the bytes figure stays for reference."""
    if "kks_newton" in roofs and kt["kks_newton"]["ms"] > 0:
        r = roofs["kks_newton"]
        r["bound"] = "issue (FP32 + MUFU per Newton iteration); bytes figure for reference"
        r["newton_iters"] = res["kks_iters_profiled"]
        r["newton_iters_per_s"] = res["kks_iters_profiled"] / (kt["kks_newton"]["ms"] / 1e3)
    return roofs


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class State:
    """Initial state of a workload: phi, c and, per model, the evolving
    quaternions or the static orientation of the anisotropic flux."""

    def __init__(self, phi, c, quat=None, orient=None):
        self.phi, self.c, self.quat, self.orient = phi, c, quat, orient

    def load(self, stepper):
        stepper.set_state(self.phi, self.c)
        if self.quat is not None:
            stepper.set_quat(self.quat)
        if self.orient is not None:
            stepper.set_orientation(self.orient)


def default_n(kind):
    return {"calphad": 256, "poly": 128, "dendrite": 2048, "dilute": 256}[kind]


def workload(n, kind="calphad", seed=3, state=True):
    """calphad: phi + c CALPHAD 3D, T_run + 50 K gradient (the headline);
    poly: phi + q + c CALPHAD polycrystal 3D at 1500 K, seeded Voronoi grains
    (8 at 128^3, 64 at 512^3), 6-cell liquid channel; dendrite: 2D dilute KKS,
    four-fold anisotropic flux (delta 0.02), undercooling 0.55, 16 seeds of
    radius 8 with random orientation angles; dilute: 2D dilute KKS at 900 K,
    isotropic nine-point flux, one tanh seed of radius 20 (width 3) in
    c = 0.02 +- 1e-3.  state=False: the model only."""
    from ampe_gb300 import configs, initial

    if kind == "dilute":
        m = configs.dilute2d(n)
        if not state:
            return m, None
        phi, c = initial.dilute2d_state(n, seed=seed, radius=20.0, width=3.0)
        return m, State(phi, c)
    if kind == "poly":
        m = configs.polycrystal3d(n, seed=seed, T=1500.0)
        if not state:
            return m, None
        ngr = max(8, (n // 128) ** 3 * 8)
        phi, c, q = initial.polycrystal_state(n, ngrains=ngr, seed=1, channel=6.0)
        return m, State(phi, c, quat=q)
    if kind == "dendrite":
        m = configs.dendrite2d(n)
        if not state:
            return m, None
        phi, c, q = initial.dendrite2d_state(n, nseeds=16, radius=8.0, seed=seed)
        return m, State(phi, c, orient=q)
    m = configs.calphad3d(n, seed=seed, T_run=1500.0)
    if not state:
        return m, None
    phi, c = initial.calphad3d_state(n, seed=seed, nseeds=max(2, (n // 32) ** 3 // 2),
                                     radius=max(4.0, n / 20.0))
    return m, State(phi, c)


WORKLOAD_NAMES = {
    "calphad": "phi+c CALPHAD implicit step %d^3 (dt=0.1, BDF<=2, Newton-GMRES(5), "
               "MG-preconditioned FAC blocks, atol %g)",
    "poly": "phi+q+c CALPHAD polycrystal implicit step %d^3 (dt=0.1, BDF<=2, "
            "Newton-GMRES(5), MG-preconditioned FAC blocks, atol %g)",
    "dendrite": "phi+c dilute anisotropic dendrite implicit step %d^2 (dt=0.1, BDF<=2, "
                "Newton-GMRES(5), MG-preconditioned FAC blocks, atol %g)",
    "dilute": "phi+c dilute isotropic implicit step %d^2 (dt=0.1, BDF<=2, "
              "Newton-GMRES(5), MG-preconditioned FAC blocks, atol %g)",
}


def step_params(args, path):
    from ampe_gb300 import configs

    return configs.step_params(dt=0.1, precond=args.precond, mg_levels=5, atol=args.atol,
                               precision=0 if path == "fp64" else 1,
                               surrogate=1 if path == "mixed+surrogate" else 0)


def cpu_sample_n(args):
    """Side of the CPU sample level: cpu_n^3 in 3D, (8 cpu_n)^2 for the 2D
    dendrite, the whole level for the small 2D dilute case."""
    if args.workload == "dilute":
        return min(args.n, 8 * args.cpu_n)
    return args.cpu_n if args.workload != "dendrite" else 8 * args.cpu_n


L2_BYTES = 129 * 10 ** 6        # GB300 L2
L2_FLUSH_BYTES = 256 * 2 ** 20  # written before each timed step of a small level


def state_fields(kind):
    return 6 if kind == "poly" else 2  # phi, c (+ four quaternion components)


def flushes_l2(args, m):
    """Levels whose state fits in L2 are timed step by step with an L2 flush
    before every step; larger ones stream their inputs from HBM anyway."""
    return m.cells() * 8 * state_fields(args.workload) < L2_BYTES


def arm_config(args, head=None, ws=1, n=None):
    """The config object of an arm's JSON line: the workload at side n (the
    full size by default; the reference arm passes the side it stepped)."""
    n = args.n if n is None else n
    m, _ = workload(n, args.workload, state=False)
    N = m.cells()
    mb = N * 8 * state_fields(args.workload) / 2 ** 20
    if flushes_l2(args, m):
        l2 = ("L2 flushed before every timed step (a %d MB write, not timed): "
              "state %.1f MB < L2" % (L2_FLUSH_BYTES // 2 ** 20, mb))
    else:
        l2 = "inputs larger than L2 (state %.0f MB)" % mb
    name = WORKLOAD_NAMES[args.workload] % (n, args.atol)
    if n != args.n:
        name += ": %d-cell sample of the %d-cell level" % (N, full_cells(args))
    path = head or args.path
    if path == "mixed+surrogate":
        path = "mixed+surrogate (network on cold starts; warm steps start from the previous step)"
    return {"workload": name, "path": path, "cells": N, "l2": l2,
            "parallelism": "replicas" if ws > 1 else "single"}


def full_cells(args):
    m, _ = workload(args.n, args.workload, state=False)
    return m.cells()


def cpu_baseline(args, threads=None):
    """The oracle on a bounded sample (cpu_n^3 level, same physics)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle as O

    n = cpu_sample_n(args)
    m, st0 = workload(n, args.workload)
    p = step_params(args, "fp64")
    s = O.OracleStepper(m, p)
    st0.load(s)
    s.advance(1)  # warm-up (first-touch, BDF1 start)
    steps = 5
    t0 = time.perf_counter()
    rc, st = s.advance(steps)
    dt = time.perf_counter() - t0
    cores = threads or os.cpu_count()
    return {"value": m.cells() * steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d cells (%s), %d implicit steps (after 1 warm-up), oracle/ C++ FP64"
                      % (m.cells(), args.workload, steps)}


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle as O

    n = cpu_sample_n(args)
    m, st0 = workload(n, args.workload)
    p = step_params(args, "fp64")
    s = O.OracleStepper(m, p)
    st0.load(s)
    s.advance(max(1, args.warmup))
    t0 = time.perf_counter()
    rc, st = s.advance(args.steps)
    dt = time.perf_counter() - t0
    v = m.cells() * args.steps / dt
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": arm_config(args, n=n),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d^%d level (%d cells) of the same workload, %d implicit "
                                   "steps per timed run, oracle/ C++ FP64 with OpenMP (reference "
                                   "sources unbuildable here: no SAMRAI/SUNDIALS/hypre/Thermo4PFM)"
                                   % (n, m.dim, m.cells(), args.steps)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def train_surrogate(args, m, local):
    """Train the KKS-guess MLP for this workload's thermodynamics on 2^22
    samples labelled by the FP64 Newton (outside the timed region)."""
    import torch

    from ampe_gb300 import _native

    L = _native.lib
    h = C.c_void_p()
    _native.check(L.ampe_mlp_create(C.byref(m), 4096, 11, C.byref(h)), "ampe_mlp_create")
    t_lo = m.T0
    t_hi = m.T0 + m.gradT * m.n[0] * m.dx[0]
    fails = C.c_longlong()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _native.check(L.ampe_mlp_generate(h, args.surrogate_samples, 99, t_lo, t_hi, 0.01, 0.99,
                                      C.byref(fails)), "ampe_mlp_generate")
    t1 = time.perf_counter()
    loss = C.c_float()
    _native.check(L.ampe_mlp_train(h, args.surrogate_steps, 4096, 3e-3, C.byref(loss)),
                  "ampe_mlp_train")
    t2 = time.perf_counter()
    info = {"samples": args.surrogate_samples, "label_newton_failures": fails.value,
            "label_s": t1 - t0, "train_steps": args.surrogate_steps, "batch": 4096,
            "train_s": t2 - t1, "final_loss": loss.value,
            "arch": "3-64-64-64-2 SiLU, BF16 weights, FP32 accumulate; inference tcgen05"}
    return h, info


def timed_path(args, m, st0, path, local, mlp=None):
    """Warm up, then time args.steps accepted steps of one path on the device.
    Returns (result dict, final host state, stepper)."""
    import torch

    from ampe_gb300 import _native
    from ampe_gb300.stepper import ImplicitStepper

    L = _native.lib
    N = m.cells()
    g = ImplicitStepper(m, step_params(args, path))
    if path == "mixed+surrogate":
        _native.check(L.ampe_stepper_attach_surrogate(g._h, mlp), "attach_surrogate")
    stream = torch.cuda.ExternalStream(L.ampe_stepper_stream(g._h))
    # cold start (no converged phase concentrations yet: the surrogate's
    # case), timed on its own after one untimed step that loads the modules
    st0.load(g)
    g.advance(1)
    st0.load(g)
    k0 = g.advance(0)["kks_iters"]
    c0 = torch.cuda.Event(enable_timing=True)
    c1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    c0.record(stream)
    cst = g.advance(1)
    c1.record(stream)
    torch.cuda.synchronize()
    cold = {"ms": c0.elapsed_time(c1), "kks_iters": cst["kks_iters"] - k0}
    g.advance(max(0, args.warmup - 1))
    torch.cuda.synchronize()
    launches0 = L.ampe_stepper_kernel_launches(g._h)
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    prof_range = args.profile_range and path == args.path
    if prof_range:
        torch.cuda.profiler.start()
    if flushes_l2(args, m):
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
        ms = 0.0
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0.record(stream)
            st = g.advance(1)
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
        del flush
    else:
        e0.record(stream)
        st = g.advance(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
    if prof_range:
        torch.cuda.profiler.stop()
    clocks.stop()
    launches = L.ampe_stepper_kernel_launches(g._h) - launches0
    # the fields at the end of the timed steps (warm-up + steps): the errors
    # between paths are reported at this step count
    state = {"phi": None, "c": None}
    state["phi"], state["c"] = g.get_state()[:2]
    if st0.quat is not None:
        state["q"] = g.get_quat()
    # per-kernel CUDA-event times in a separate pass of the same number of
    # steps (events around every kernel class and a stream synchronisation
    # per step), so that the timed steps above carry no instrumentation
    L.ampe_stepper_profile(g._h, 1)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    p0.record(stream)
    st_prof = g.advance(args.steps)
    p1.record(stream)
    torch.cuda.synchronize()
    ms_prof = p0.elapsed_time(p1)
    kt = {}
    for kind, name in KINDS:
        tot, cnt = C.c_double(), C.c_longlong()
        L.ampe_stepper_kernel_time(g._h, kind, C.byref(tot), C.byref(cnt))
        kt[name] = {"ms": tot.value, "launches": cnt.value}
    L.ampe_stepper_profile(g._h, 0)
    return {"ms": ms, "ms_profiled": ms_prof, "stats": st, "launches": int(launches),
            "kks_iters_profiled": st_prof["kks_iters"] - st["kks_iters"],
            "kernels": kt,
            "clocks": clocks.summary(), "value": N * args.steps / (ms / 1e3),
            "cold_start_step": cold}, state, g


def surrogate_study(args, m, st0, mlp):
    """Newton iterations per cell and KKS solve, surrogate fallback rate and
    wall time of args.surrogate_study_steps steps from the cold initial
    state, for the mixed path with the plain warm start (the previous
    step's phase concentrations, QuatModel.cc:5218-5231), with the network's
    guess on cold starts only, and with the network's guess for every KKS
    solve (the warm start then only the fallback)."""
    import torch

    from ampe_gb300 import _native, configs
    from ampe_gb300.stepper import ImplicitStepper

    L = _native.lib
    n = args.surrogate_study_steps
    out = {"steps": n, "cells": m.cells(),
           "start": "the workload's initial state without phase concentrations (cold)"}
    for name, mode in (("warm_start", 0), ("surrogate_cold_start", 1),
                       ("surrogate_every_solve", 2)):
        p = configs.step_params(dt=0.1, precond=args.precond, mg_levels=5, atol=args.atol,
                                precision=1, surrogate=mode)
        g = ImplicitStepper(m, p)
        if mode:
            _native.check(L.ampe_stepper_attach_surrogate(g._h, mlp), "attach_surrogate")
        stream = torch.cuda.ExternalStream(L.ampe_stepper_stream(g._h))
        st0.load(g)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        st = g.advance(n)
        e1.record(stream)
        torch.cuda.synchronize()
        solves = m.cells() * st["rhs_evals"]
        out[name] = {"wall_s": e0.elapsed_time(e1) / 1e3,
                     "kks_newton_iters_per_cell_solve": st["kks_iters"] / solves,
                     "fallback_rate": st["kks_fallback"] / solves,
                     "kks_failed_cells": st["kks_fail"], "rhs_evals": st["rhs_evals"],
                     "newton_iters": st["newton_iters"]}
        g.close()
        del g
        torch.cuda.empty_cache()
    return out


def run_ours(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from ampe_gb300 import _native

    L = _native.lib
    m, st0 = workload(args.n, args.workload)
    N = m.cells()
    head = args.path
    mlp, sur_info = None, None
    if head == "mixed+surrogate":
        mlp, sur_info = train_surrogate(args, m, local)
    if ws > 1:
        dist.barrier()
    res_h, st_h, g = timed_path(args, m, st0, head, local, mlp)
    ms_max, updates = aggregate(res_h["ms"], N * args.steps)
    value = updates / (ms_max / 1e3)

    # end to end through the C-ABI, state from pinned host memory each step
    e2e = None
    if not args.no_e2e and args.workload == "calphad":
        hp = torch.empty(N, dtype=torch.float64).pin_memory()
        hc = torch.empty(N, dtype=torch.float64).pin_memory()
        L.ampe_stepper_get_state(g._h, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()),
                                 None, None, 1)
        ke = max(2, min(args.steps, 6))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(ke):
            L.ampe_stepper_load_y(g._h, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()), 1)
            g.advance(1)
            L.ampe_stepper_get_state(g._h, C.c_void_p(hp.data_ptr()), C.c_void_p(hc.data_ptr()),
                                     None, None, 1)
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        te_max, upd_e = aggregate(te * 1e3, N * ke)
        e2e = {"value": upd_e / (te_max / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": 2 * N * 8, "d2h_bytes_per_step": 2 * N * 8,
               "steps": ke}
    g.close()
    del g
    torch.cuda.empty_cache()

    # the other paths on the same input: speed ratios and errors vs FP64
    results = {head: (res_h, st_h)}
    for other in ("mixed", "fp64", "mixed+surrogate"):
        if other in results or args.only_head:
            continue
        if other == "mixed+surrogate" and mlp is None:
            continue
        r, st, g2 = timed_path(args, m, st0, other, local, mlp)
        g2.close()
        del g2
        torch.cuda.empty_cache()
        results[other] = (r, st)
    paths = {}
    ref = results.get("fp64")
    for name, (r, st) in results.items():
        d = {"value": r["value"], "ms_per_step": r["ms"] / args.steps,
             "kks_iters": r["stats"]["kks_iters"], "kks_fallback": r["stats"]["kks_fallback"],
             "newton_iters": r["stats"]["newton_iters"], "gmres_iters": r["stats"]["gmres_iters"],
             "clocks": r["clocks"], "kernels_ms": {k: v["ms"] for k, v in r["kernels"].items()
                                                   if v["launches"]},
             "cold_start_step": r["cold_start_step"]}
        if ref is not None and name != "fp64":
            d["speedup_vs_fp64"] = r["value"] / ref[0]["value"]
            d["rel_l2_err_vs_fp64"] = {
                f: float(np.linalg.norm((st[f] - ref[1][f]).ravel())
                         / np.linalg.norm(ref[1][f].ravel()))
                for f in st}
        paths[name] = d
    if args.ref_atol > 0.0:
        # untimed reference: FP64 path at a tighter Newton tolerance; the
        # error of each path against it compares with its own tolerance error
        from ampe_gb300.stepper import ImplicitStepper
        from ampe_gb300 import configs

        pr = configs.step_params(dt=0.1, precond=args.precond, mg_levels=5, atol=args.ref_atol,
                                 precision=0)
        gr = ImplicitStepper(m, pr)
        st0.load(gr)
        gr.advance(args.warmup + args.steps)  # the step count the paths are compared at
        refs = {"phi": None, "c": None}
        refs["phi"], refs["c"] = gr.get_state()[:2]
        if st0.quat is not None:
            refs["q"] = gr.get_quat()
        gr.close()
        for name, (r, st) in results.items():
            paths[name]["rel_l2_err_vs_fp64_atol_%g" % args.ref_atol] = {
                f: float(np.linalg.norm((st[f] - refs[f]).ravel())
                         / np.linalg.norm(refs[f].ravel()))
                for f in st}
    study = None
    if mlp is not None and args.surrogate_study_steps > 0 and args.workload == "calphad":
        study = surrogate_study(args, m, st0, mlp)
    if mlp is not None:
        L.ampe_mlp_destroy(mlp)

    pk, pk_kind = peaks()
    # dominant instrumented kernel of the headline path and its roofline
    kt = res_h["kernels"]
    per_cell = {"kks_newton": KKS_BYTES_PER_CELL if head == "fp64" else KKS_MIXED_BYTES_PER_CELL,
                "rhs_fused": RHS_BYTES_PER_CELL if head == "fp64" else RHS_MIXED_BYTES_PER_CELL,
                "jv_analytic": JV_BYTES_PER_CELL,
                "smooth_fine": SMOOTH_BYTES_PER_CELL_FP64[m.dim] if head == "fp64"
                else SMOOTH_BYTES_PER_CELL[m.dim]}
    kname = max((k for k in SINGLE_KERNELS if kt[k]["launches"]), key=lambda k: kt[k]["ms"])
    tot, cnt = kt[kname]["ms"], kt[kname]["launches"]
    avg_ms = tot / max(cnt, 1)
    if kname == "mlp_infer_tc":
        flops = MLP_FLOPS_PER_CELL * N
        achieved = flops / (avg_ms / 1e3) / 1e12
        roof = {"bound": "tensor", "kernel": "k_mlp_infer_tc", "achieved": achieved,
                "peak": pk["bf16_tflops"], "peak_kind": pk_kind, "unit": "TFLOP/s",
                "frac": achieved / pk["bf16_tflops"], "traffic": None,
                "algorithmic_flops_per_launch": flops}
    else:
        nbytes = per_cell[kname] * N
        achieved = nbytes / (avg_ms / 1e3) / 1e9
        kn = KERNEL_NAMES[head == "fp64"][kname]
        if isinstance(kn, dict):
            kn = kn[m.dim]
        traffic = None
        if (kname == "smooth_fine" and head != "fp64" and args.workload == "calphad"
                and SMOOTH_DRAM_BYTES_PER_CELL_MEASURED is not None):
            traffic = SMOOTH_DRAM_BYTES_PER_CELL_MEASURED * N
        roof = {"bound": "hbm", "kernel": kn,
                "achieved": achieved, "peak": pk["hbm_gbs"], "peak_kind": pk_kind, "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": traffic,
                "algorithmic_bytes_per_launch": nbytes}
        if traffic is not None:
            roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of both "
                                      "blocks' colour launches at 224^3, scaled by cells")
    roof.update({"avg_launch_ms": avg_ms, "launches": cnt,
                 "share_of_step": tot / res_h["ms_profiled"],
                 "timing": "kernel times from a profiled pass of %d further steps (%.2f ms/step "
                           "with the per-kernel events, %.2f ms/step without)"
                           % (args.steps, res_h["ms_profiled"] / args.steps,
                              res_h["ms"] / args.steps)})
    if sur_info is not None:
        # whether the network ran inside the timed steps: it is evaluated only
        # while no converged warm start exists (a cold start)
        sur_info["inferences_in_timed_steps"] = kt["mlp_infer_tc"]["launches"]
        if not kt["mlp_infer_tc"]["launches"]:
            sur_info["timed_steps"] = (
                "the network is not evaluated in the timed (warm) steps: the previous step's "
                "phase concentrations start the KKS Newton in fewer iterations than its guess; "
                "it starts cold steps only (cold_start_step, surrogate_study)")
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if head == "fp64" else "f32+f64",
        "data": "synthetic",
        "config": arm_config(args, head, ws),
        "paths": paths,
        "surrogate": sur_info,
        "surrogate_study": study,
        "roofline": roof,
        "kernel_rooflines": kks_issue(kernel_rooflines(kt, per_cell, N, pk), kt, res_h),
        "kernels": res_h["kernels"],
        "stats": res_h["stats"],
        "gpu_launches": res_h["launches"],
        "clocks": res_h["clocks"],
        "e2e": e2e,
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.n <= 0:
        args.n = default_n(args.workload)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
