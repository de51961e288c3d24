#!/usr/bin/env python
"""Benchmark: MCTDHF trajectory-steps/s on one GB300.

One step = one Strang split step Propagate(t, t+dt): short-iterative-Lanczos
half steps on the one-body part (fixed Krylov order, grid-weighted metric)
around an RK4 step of the nonlinear part (CI H.C, RDMs, pair potentials,
mean-field contraction, (1-P) projector).

Default workload: three soft-Coulomb nuclei, FEDVR 400 elements x 8 points on
[-400, 400] (2801 points), N=6 fermions in 16 spin-orbitals (8008
determinants), dt = 0.02, Krylov order 16, sin^2 laser pulse E0 = 0.0755 au.
Synthetic seeded inputs: Gaussian orbitals (seed 7) and random normalised CI
coefficients (the step cost does not depend on the values).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MCTDHF traj-steps/s: mixed-prec batched vs FP64 GPU at ≤1e-8 energy/norm err"
UNIT = "traj-steps/s"
L2_BYTES = 129 * 1024 * 1024


def workload(name: str):
    from codyfortran_gb300 import spec as S
    if name == "trimer_large":
        return S.cfg_trimer_large(), dict(dt=0.02, krylov=16, seed=7)
    if name == "helium_small":
        return S.cfg_helium_small(), dict(dt=0.01, krylov=12, seed=42)
    raise SystemExit(f"unknown workload {name}")


def initial_state(sp, x, w, seed):
    from codyfortran_gb300 import init as I
    rng = np.random.default_rng(seed)
    orbs = I.seeded_gaussian_orbitals(sp, x, w, seed)
    c = rng.normal(size=sp.n_coeffs) + 1j * rng.normal(size=sp.n_coeffs)
    c /= np.linalg.norm(c)
    return I.pack_state(c, orbs)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out["sm_mhz"] = float(np.median(sm))
            out["sm_max_mhz"] = float(max(smax))
        out["reasons"] = sorted(reasons)
        out["samples"] = len(sm)
        return out


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_max(value: float, world: int) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(sp, cfg, state, n_threads, budget_s=25.0, max_steps=None):
    """Strang steps of the oracle (CPU port) on the host cores: bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    o = Oracle(sp, n_threads=n_threads)
    m = o.metric_weights()
    st = state.copy()
    t = 0.0
    steps, t0 = 0, time.perf_counter()
    while True:
        st = o.propagate_split2(st, t, t + cfg["dt"], krylov_dim=cfg["krylov"], metric=m)
        t += cfg["dt"]
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s or (max_steps and steps >= max_steps):
            break
    return steps, el


def run_reference(args):
    """The reference's algorithm on the host CPU (the oracle port; the Fortran reference cannot be built here)."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    sp, cfg = workload(args.workload)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    o = Oracle(sp, n_threads=os.cpu_count())
    st = initial_state(sp, o.x, o.w, cfg["seed"])
    m = o.metric_weights()
    t = 0.0
    tw0 = time.perf_counter()
    warm = 0
    for _ in range(max(args.warmup, 1)):
        st = o.propagate_split2(st, t, t + cfg["dt"], krylov_dim=cfg["krylov"], metric=m)
        t += cfg["dt"]
        warm += 1
        if time.perf_counter() - tw0 > 60.0:
            break
    per = (time.perf_counter() - tw0) / warm
    k = max(1, min(args.steps, int(120.0 / max(per, 1e-9))))
    t0 = time.perf_counter()
    for _ in range(k):
        st = o.propagate_split2(st, t, t + cfg["dt"], krylov_dim=cfg["krylov"], metric=m)
        t += cfg["dt"]
    el = time.perf_counter() - t0
    val = k / el
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
        "warmup": warm, "ms_per_step": 1e3 * el / k, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "complex128", "data": "synthetic",
        "config": {"workload": args.workload, "n_grid": o.nG, "n_determinants": o.nC, "krylov_order": cfg["krylov"],
                   "dt": cfg["dt"], "form": "CPU port of the reference algorithm (FP64)"},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{k} Strang steps of {args.workload} on {os.cpu_count()} host threads"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local)) if world > 1 else None
    from codyfortran_gb300.engine import Engine
    from codyfortran_gb300 import build as B
    B.build()
    sp, cfg = workload(args.workload)
    precision = args.precision
    e = Engine(sp, precision=precision, max_krylov=cfg["krylov"])
    st = initial_state(sp, e.x, e.w, cfg["seed"])
    dt, K = cfg["dt"], cfg["krylov"]
    e.upload(st)
    t = 0.0
    graph = not args.no_graph
    e.propagate_resident(t, dt, args.warmup, K, use_metric=True, use_graph=graph)
    t += args.warmup * dt
    e.synchronize()
    # dominant kernel: the family with the largest device time in one step (CUDA events
    # around each of its launches, recorded on the library's stream; inside the graph
    # they are event-record nodes, so the times are those of the last replayed step)
    fam_ms = {}
    for fam in ("pair_potentials", "correlation", "h2", "ci_apply", "ci_rdm", "onebody", "lanczos"):
        e.profile_begin(fam)
        e.propagate_resident(t, dt, 1, K, use_metric=True, use_graph=graph)
        t += dt
        n, ms = e.profile_end()
        fam_ms[fam] = (n, ms)
    dom = max(fam_ms, key=lambda k: fam_ms[k][1])
    e.profile_begin(dom)
    e.propagate_resident(t, dt, 1, K, use_metric=True, use_graph=graph)  # capture with the events, untimed
    t += dt
    # timed region
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    e.launch_count(reset=True)
    with ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]) if world > 1 else 0) as clk:
        ms = e.propagate_resident_timed(t, dt, args.steps, K, use_metric=True, use_graph=graph)
    n_dom, ms_dom = e.profile_end()
    launches = e.launch_count()
    t += args.steps * dt
    ms = barrier_max(ms, world)
    value = world * args.steps / (ms / 1e3)
    # end-to-end through the host-buffer C-ABI call (H2D + step + D2H per step)
    host = e.download()
    n_e2e = max(1, min(args.steps, 20))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    te0 = time.perf_counter()
    for _ in range(n_e2e):
        host = e.propagate_split2(host, t, t + dt, krylov_dim=K, use_metric=True)
        t += dt
    te = barrier_max(time.perf_counter() - te0, world)
    e2e = world * n_e2e / te
    # roofline of the dominant kernel
    hbm, bf16, src = measured_peaks()
    nG, P, Q, nC = e.nG, e.nOS * (e.nOS + 1) // 2, e.nOS * e.nOS, e.nC
    avg_s = (ms_dom / max(n_dom, 1)) / 1e3
    if dom == "pair_potentials":
        work, bound = 2.0 * nG * nG * 2 * P, "tensor"       # W = V S, real GEMM nG x nG x 2P
    elif dom in ("correlation", "h2"):
        work, bound = 8.0 * nG * Q * Q, "tensor"            # complex GEMM nG x Q x Q
    else:
        work, bound = 16.0 * e.nS * 4, "hbm"                # streaming estimate
    if bound == "tensor":
        achieved, peak, unit = work / avg_s / 1e12, bf16, "TFLOP/s"
    else:
        achieved, peak, unit = work / avg_s / 1e9, hbm, "GB/s"
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "complex128" if precision == "fp64" else "mixed(bf16x3/fp32 contractions, fp64 rest)",
        "data": "synthetic (seeded Gaussian orbitals, random normalised CI vector)",
        "config": {"workload": args.workload, "n_grid": nG, "n_orbitals": e.nOS, "n_determinants": nC,
                   "krylov_order": K, "dt": dt, "precision": precision, "parallelism": f"replicas x{world}",
                   "l2": f"per-step working set {(nG * nG * 8 + 71e6 + (K + 8) * e.nS * 16) / 1e6:.0f} MB > L2 "
                         f"({L2_BYTES / 1e6:.0f} MB): inputs larger than L2, no flush"},
        "clocks": clocks,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": e.nS * 16, "d2h_bytes_per_step": e.nS * 16,
                "steps": n_e2e, "call": "cgpu_propagate_split2 (host state in/out)"},
        "gpu_launches": int(launches),
        "roofline": {"kernel": dom, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
                     "frac": achieved / peak, "peak_source": src, "traffic": None,
                     "launches": n_dom, "avg_launch_us": avg_s * 1e6, "work_per_launch": work},
        "kernel_ms_per_step": {k: v[1] for k, v in fam_ms.items()},
    }
    if rank == 0 and not args.no_cpu_baseline:
        steps_cpu, el = cpu_sample(sp, cfg, st, os.cpu_count(), budget_s=args.cpu_budget, max_steps=3)
        line["cpu_baseline"] = {"value": steps_cpu / el, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{steps_cpu} Strang step(s) of {args.workload} ({el:.1f} s)"}
    if rank == 0:
        print(json.dumps(line))
    e.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="trimer_large")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "mixed6"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=25.0)
    ap.add_argument("--no-graph", action="store_true", help="launch kernels one by one instead of a step graph")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
