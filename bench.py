#!/usr/bin/env python
"""Benchmark: MCTDHF trajectory-steps/s on one GB300.

One trajectory-step = one Strang split step Propagate(t, t+dt) of one
trajectory: short-iterative-Lanczos half steps on the one-body part (fixed
Krylov order, grid-weighted metric) around an RK4 step of the nonlinear part
(CI H.C, RDMs, pair potentials, mean-field contraction, (1-P) projector).

Default workload (batch512): 512 independent 1D soft-Coulomb MCTDHF
trajectories drawn from seed 1234 -- N in {2,4} electrons as two restricted
spin body types, M uniform in 4..12 spatial orbitals, FEDVR 100..400 elements
x 6 points on [-nE, nE], sin^2 4-cycle pulses at omega = 0.057 au with
log-uniform intensity 1e13..1e15 W/cm^2 and uniform CEP; dt = 0.02, Krylov
order 12; mixed precision mixed_fx6 (the pair-potential, correlation and h2
contractions on tcgen05 tensor cores with every operand row carried as digit
slices holding 36 bits of the row maximum -- six base-64 slices on the grid
contractions, five base-256 slices on the pair contraction -- and exact
per-level accumulation; FP64 elsewhere; three-term Lanczos recurrence).  The
faster mixed_fx form (30 bits) is selected with --precision mixed_fx.
All trajectories advance together: every kernel of the step covers the whole
batch and the step is one CUDA-graph launch.  The same batch in the plain FP64
form is timed beside it (the "vs FP64 GPU" leg of the metric).

Other workload: trimer_large -- three soft-Coulomb nuclei, FEDVR 400 x 8
points on [-400, 400] (2801 points), N=6 fermions in 16 spin-orbitals (8008
determinants), dt = 0.02, Krylov order 16, E0 = 0.0755 au.

Synthetic seeded inputs: Gaussian orbitals and random normalised CI
coefficients (the step cost does not depend on the values).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload batch512|trimer_large|helium_small]
                  [--precision fp64|mixed|mixed6|mixed_fx|mixed_fx6]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MCTDHF traj-steps/s: mixed-prec batched vs FP64 GPU at ≤1e-8 energy/norm err"
UNIT = "traj-steps/s"
L2_BYTES = 129 * 1024 * 1024
ACC_STEPS = 10
ACC_STEPS_SINGLE = 20
DTYPES = {
    "fp64": "complex128",
    "mixed": "mixed (bf16x3 tcgen05 contractions with fp32 accumulation, fp64 rest)",
    "mixed6": "mixed (bf16x6 tcgen05 contractions with fp32 accumulation, fp64 rest)",
    "mixed_fx": "mixed (tcgen05 contractions on bf16 digit slices holding 30 bits of each operand row's maximum: "
                "5 base-64 slices for K = n_grid, 4 base-256 for K = 2 n_pairs; exact per-level accumulation, "
                "fp64 results; fp64 rest)",
    "mixed_fx6": "mixed (tcgen05 contractions on bf16 digit slices holding 36 bits of each operand row's maximum: "
                 "6 base-64 slices for K = n_grid, 5 base-256 for K = 2 n_pairs; exact per-level accumulation, "
                 "fp64 results; fp64 rest)",
}
FAMILIES = ("pair_potentials", "correlation", "h2", "ci_apply", "ci_rdm", "onebody", "lanczos", "rdm_inverse",
            "projectors", "fold", "vector")


def workload(name: str):
    from codyfortran_gb300 import spec as S
    if name == "batch512":
        return S.batch_trajectory_specs(512, 1234), dict(dt=0.02, krylov=12, seed=1234)
    if name == "trimer_large":
        return [S.cfg_trimer_large()], dict(dt=0.02, krylov=16, seed=7)
    if name == "helium_small":
        return [S.cfg_helium_small()], dict(dt=0.01, krylov=12, seed=42)
    raise SystemExit(f"unknown workload {name}")


def initial_state(sp, x, w, seed):
    from codyfortran_gb300 import init as I
    rng = np.random.default_rng(seed)
    orbs = I.seeded_gaussian_orbitals(sp, x, w, seed)
    c = rng.normal(size=sp.n_coeffs) + 1j * rng.normal(size=sp.n_coeffs)
    c /= np.linalg.norm(c)
    return I.pack_state(c, orbs)


def measured_peaks(sustained=False):
    """(HBM GB/s, bf16 TFLOP/s, source).  sustained: the bf16 figure of a
    seconds-long GEMM loop under the power cap, the denominator for a kernel
    timed inside a long step; otherwise the burst figure."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        key = "bf16_tflops_sustained" if sustained and "bf16_tflops_sustained" in d else "bf16_tflops"
        return d.get("hbm_gbs", 6800.0), d.get(key, 1900.0), f"measured ({key})"
    return 6800.0, 1700.0 if sustained else 1900.0, "fallback"


def cpu_model():
    """The host CPU's model name (lscpu / /proc/cpuinfo), or the machine type."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


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


def oracle_traj_steps(specs, cfg, n_threads, budget_s, max_traj=None):
    """Strang steps of the oracle (the CPU port of the reference algorithm) on the
    host cores, over the first trajectories of the workload: returns (steps, seconds, trajectories)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    steps, el, used = 0, 0.0, 0
    t_start = time.perf_counter()
    for k, sp in enumerate(specs[:max_traj] if max_traj else specs):
        o = Oracle(sp, n_threads=n_threads)
        m = o.metric_weights()
        st = initial_state(sp, o.x, o.w, cfg["seed"] + k)
        t = 0.0
        t0 = time.perf_counter()
        n = 0
        while True:
            st = o.propagate_split2(st, t, t + cfg["dt"], krylov_dim=cfg["krylov"], metric=m)
            t += cfg["dt"]
            n += 1
            if time.perf_counter() - t0 > budget_s / max(1, min(len(specs), 8)) or n >= 3:
                break
        el += time.perf_counter() - t0
        steps += n
        used += 1
        if time.perf_counter() - t_start > budget_s:
            break
    return steps, el, used


def _oracle_traj_worker(job):
    """One trajectory of the CPU port on one host core: set-up and one untimed
    step, then `steps` timed Strang steps.  Returns (steps, seconds)."""
    sp, seed, dt, K, steps = job
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, ROOT)
    from oracle import Oracle
    o = Oracle(sp, n_threads=1)
    m = o.metric_weights()
    st = initial_state(sp, o.x, o.w, seed)
    st = o.propagate_split2(st, 0.0, dt, krylov_dim=K, metric=m)
    t = dt
    t0 = time.perf_counter()
    for _ in range(steps):
        st = o.propagate_split2(st, t, t + dt, krylov_dim=K, metric=m)
        t += dt
    return steps, time.perf_counter() - t0


def oracle_parallel_traj_steps(specs, cfg, n_workers, n_sample=64, steps=2):
    """Trajectory-parallel throughput of the CPU port: a sample of n_sample
    trajectories spread evenly over the workload (every len/n_sample-th), one
    trajectory per worker process and host core (one OpenMP thread each),
    largest first.  Throughput = n_workers x (timed steps / summed
    single-core seconds), the rate of n_workers cores that stay busy.
    Returns (value, dict describing the sample)."""
    import multiprocessing as mp
    stride = max(1, len(specs) // n_sample)
    idx = list(range(0, len(specs), stride))[:n_sample]
    cost = lambda sp: sp.n_grid ** 2 * sp.n_orbs[0] ** 2 + sp.n_grid * sp.n_orbs[0] ** 4
    idx.sort(key=lambda i: -cost(specs[i]))
    jobs = [(specs[i], cfg["seed"] + i, cfg["dt"], cfg["krylov"], steps) for i in idx]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(n_workers) as pool:
        res = pool.map(_oracle_traj_worker, jobs, chunksize=1)
    wall = time.perf_counter() - t0
    n_steps = sum(r[0] for r in res)
    core_s = sum(r[1] for r in res)
    value = n_workers * n_steps / core_s
    return value, {"trajectories": len(idx), "steps_per_trajectory": steps, "timed_steps": n_steps,
                   "core_seconds": core_s, "wall_seconds": wall}


def run_reference(args):
    """The reference's algorithm on the host CPU (the oracle port; the Fortran
    reference cannot be built in this environment), on the workload's trajectories."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    specs, cfg = workload(args.workload)
    cores = os.cpu_count()
    if len(specs) > 1:
        val, smp = oracle_parallel_traj_steps(specs, cfg, cores)
        steps, el = smp["timed_steps"], smp["core_seconds"] / cores
        form = "CPU port of the reference algorithm (FP64), one trajectory per host core"
        sample = (f"{smp['timed_steps']} Strang steps over {smp['trajectories']} trajectories spread over "
                  f"{args.workload} ({smp['steps_per_trajectory']} timed steps each after one untimed), one "
                  f"trajectory per worker process on {cores} cores of {cpu_model()}: {cores} x steps / "
                  f"{smp['core_seconds']:.1f} summed core-seconds ({smp['wall_seconds']:.1f} s wall)")
    else:
        steps, el, used = oracle_traj_steps(specs, cfg, cores, 60.0)
        val = steps / el
        form = "CPU port of the reference algorithm (FP64), one trajectory on all host threads"
        sample = f"{steps} Strang steps of {args.workload} on {cores} host threads of {cpu_model()}"
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": 0, "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "complex128", "data": "synthetic (seeded Gaussian orbitals, random CI vector)",
        "config": {"workload": args.workload, "trajectories": len(specs), "krylov_order": cfg["krylov"],
                   "dt": cfg["dt"], "form": form},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(),
                         "sample": sample},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def lanczos_work(systems, K, window=0, sil_per_step=2):
    """Algorithmic bytes and FP64 flops of the Lanczos family in one step.  At
    iteration j the update forms the dots of w with the nv basis vectors it
    orthogonalises against (nv = j, or min(j, window)) and ||w||^2 (reads nv + 1
    vectors and the metric), subtracts the projections and forms the new norm
    (reads nv + 1 vectors and the metric, writes w) and scales w into v_{j+1}
    (reads w, writes v_{j+1}): (2 nv + 5) complex and 2 real passes over the
    state; 16 nv + 13 flops per entry.  The three-term recurrence (window 1)
    reads v_{j-1}, v_j, w twice (one real dot and ||w||^2, then the update with
    the new norm), writes w, then scales: 8 complex and 2 real passes, 28 flops
    per entry.  The gated second pass does not fire on this workload and is not
    counted."""
    nS = sum(s.nS for s in systems)
    if window == 1:
        per = [(16.0 * 8 + 16.0, 28) for _ in range(1, K + 1)]
    else:
        nvs = [min(j, window) if window > 0 else j for j in range(1, K + 1)]
        per = [(16.0 * (2 * nv + 5) + 16.0, 16 * nv + 13) for nv in nvs]
    byts = sum(b for b, _ in per) * sil_per_step * nS
    flops = sum(f for _, f in per) * sil_per_step * nS
    return byts, float(flops)


def dense_flops(systems, fam):
    """Algorithmic flops of one NonLin evaluation's dense contraction (four per step)."""
    tot = 0.0
    for s in systems:
        n = s.nOS
        P = n * (n + 1) // 2
        if fam == "pair_potentials":
            tot += 4.0 * s.nG * s.nG * P
        elif fam in ("correlation", "h2"):
            tot += 8.0 * s.nG * n ** 4
    return 4.0 * tot


FX_BITS = {"mixed_fx": 30, "mixed_fx6": 36}

# DRAM bytes per launch of the dominant family, from one full-size ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum over the family's kernels of
# one evaluation; the summary and its command are in the named file)
PROFILED_TRAFFIC = {
    # 32-trajectory capture scaled by the units processed (a lower bound: the
    # small case keeps the digit planes in L2)
    ("batch512", "mixed_fx6", "pair_potentials"): (5.82e9, "profiles/dram_traffic_pair_potentials_fx6_batch32.md"),
}


def fx_grid_products(precision, systems):
    """Slice products per algorithmic product of the fixed-point contractions
    over the grid: digit width b = 8 / 7 / 6 for K <= 256 / 1024 / longer (the
    two leading level sums stay exact in FP32), L = ceil(bits / b) slices and
    the L (L + 1) / 2 slice products of the levels below L."""
    K = max(s.nG for s in systems)
    b = 8 if K <= 256 else 7 if K <= 1024 else 6
    L = -(-FX_BITS[precision] // b)
    return L * (L + 1) // 2


def systems_of(r):
    return r["systems"]


def batch_norms(b, packed):
    """||C|| of every trajectory (orthonormal orbitals: the MCTDHF norm)."""
    return np.array([np.linalg.norm(packed[b.offsets[i]:b.offsets[i] + b.systems[i].nC]) for i in range(len(b))])


def run_batch_leg(specs, cfg, precision, steps, warmup, profile=True, clock=False, e2e=True, acc_steps=0, window=0,
                  tune=True):
    from codyfortran_gb300.engine import Batch, pinned_empty
    dt, K = cfg["dt"], cfg["krylov"]
    b = Batch(specs, precision, max_krylov=K, krylov_window=window)
    states = [initial_state(sp, s.x, s.w, cfg["seed"] + k) for k, (sp, s) in enumerate(zip(specs, b.systems))]
    host = b.pack(states)
    b.upload(host)
    tiles = None
    if tune:
        # the project's tile autotuner on the batch's own shapes (outside the timed region)
        t0 = time.perf_counter()
        heuristic = b.tiles()
        rep = b.autotune()
        tiles = {"tiles": "autotuned", "source": rep["source"], "table": rep["tiles"], "heuristic": heuristic,
                 "seconds": time.perf_counter() - t0}
        b.upload(host)
    t = 0.0
    b.propagate(t, dt, warmup, K)
    t += warmup * dt
    fam_ms = {}
    if profile:
        for fam in FAMILIES:
            b.profile_begin(fam)
            b.propagate(t, dt, 1, K)
            t += dt
            fam_ms[fam] = b.profile_end()
    dom = max(fam_ms, key=lambda k: fam_ms[k][1]) if fam_ms else None
    if dom:
        b.profile_begin(dom)
        b.propagate(t, dt, 1, K)  # capture the graph with the dominant family's events, untimed
        t += dt
    b.launch_count(reset=True)
    clk = ClockSampler(0) if clock else None
    if clk:
        clk.__enter__()
    ms = b.propagate(t, dt, steps, K)
    if clk:
        clk.__exit__()
    t += steps * dt
    n_dom, ms_dom = b.profile_end() if dom else (0, 0.0)
    launches = b.launch_count()
    out = dict(ms=ms, fam_ms=fam_ms, dom=dom, n_dom=n_dom, ms_dom=ms_dom, launches=launches,
               clocks=clk.summary() if clk else None, systems=b.systems, kps=b.kernels_per_step(), tiles=tiles)
    if e2e:
        # end to end through the C ABI: packed host states in, one step, packed
        # states out, from and to page-locked host memory (cgpu_host_alloc)
        n_e2e = max(3, min(steps, 10))
        buf = pinned_empty(host.size)
        buf[:] = host
        # untimed: the step graph is re-captured without the profiling events
        b.propagate(t, dt, 1, K)
        t += dt
        te0 = time.perf_counter()
        for _ in range(n_e2e):
            b.upload(buf)
            b.propagate(t, dt, 1, K)
            b.download_packed(buf)
            t += dt
        out["e2e_s"] = (time.perf_counter() - te0) / n_e2e
        out["e2e_bytes"] = int(buf.nbytes)
    if acc_steps:
        # accuracy leg: acc_steps steps from the initial states, energies and norms at the end
        b.upload(host)
        b.propagate(0.0, dt, acc_steps, K)
        out["acc_energy"] = b.energies(acc_steps * dt)
        out["acc_norm"] = batch_norms(b, b.download_packed())
    b.close()
    return out


def accuracy_horizon(specs, cfg, precision, n_steps, every=10, window=1):
    """Deviation of a mixed-precision batch from the same batch in the FP64 form
    (the reference's full Krylov loop), both advanced from the same states for
    n_steps steps: every `every` steps the per-trajectory relative energy
    deviation |E_mixed - E_fp64| / |E_fp64|, the absolute one |E_mixed - E_fp64|
    (Hartree), the one against max(|E_fp64|, 1 Hartree) and the norm deviation
    | ||C_mixed|| - ||C_fp64|| |.  Returns rows (step, max, median, p99 of the
    relative energy deviation, max norm deviation, trajectory of the max,
    |E_fp64| of that trajectory, max absolute deviation, max deviation against
    max(|E|, 1))."""
    from codyfortran_gb300.engine import Batch
    K, dt = cfg["krylov"], cfg["dt"]
    f = Batch(specs, "fp64", max_krylov=K, krylov_window=0)
    m = Batch(specs, precision, max_krylov=K, krylov_window=window)
    states = [initial_state(sp, s.x, s.w, cfg["seed"] + k) for k, (sp, s) in enumerate(zip(specs, f.systems))]
    host = f.pack(states)
    f.upload(host)
    m.upload(host)
    rows, t = [], 0.0
    for step in range(every, n_steps + 1, every):
        f.propagate(t, dt, every, K)
        m.propagate(t, dt, every, K)
        t += every * dt
        ef, em = f.energies(t), m.energies(t)
        da = np.abs(em - ef)
        de = da / np.abs(ef)
        dn = np.abs(batch_norms(m, m.download_packed()) - batch_norms(f, f.download_packed()))
        w = int(np.argmax(de))
        rows.append((step, float(de.max()), float(np.median(de)), float(np.quantile(de, 0.99)), float(dn.max()), w,
                     float(abs(ef[w])), float(da.max()), float((da / np.maximum(np.abs(ef), 1.0)).max())))
    f.close()
    m.close()
    return rows


def run_accuracy_horizon(args):
    """--accuracy-horizon N: the per-step deviation table of accuracy_horizon on the
    first --accuracy-trajectories trajectories of the workload, as one JSON line."""
    specs, cfg = workload(args.workload)
    precision = args.precision or "mixed_fx6"
    n = min(args.accuracy_trajectories, len(specs))
    from codyfortran_gb300 import build as B
    B.build()
    t0 = time.perf_counter()
    rows = accuracy_horizon(specs[:n], cfg, precision, args.accuracy_horizon, args.accuracy_every,
                            krylov_window(args, precision))
    print(json.dumps({"mode": "accuracy_horizon", "workload": args.workload, "precision": precision,
                      "trajectories": n, "steps": args.accuracy_horizon, "dt": cfg["dt"], "krylov_order": cfg["krylov"],
                      "energy_rel_max": max(r[1] for r in rows), "norm_abs_max": max(r[4] for r in rows),
                      "energy_abs_max": max(r[7] for r in rows), "energy_rel_floor1_max": max(r[8] for r in rows),
                      "seconds": time.perf_counter() - t0,
                      "columns": ["step", "energy_rel_max", "energy_rel_median", "energy_rel_p99", "norm_abs_max",
                                  "worst_trajectory", "worst_abs_energy", "energy_abs_max", "energy_rel_floor1_max"],
                      "rows": rows}))
    return 0


def adjoint_start_state(kind, x, w, eng_relax=None):
    """Start (and reference) state of the pulse-gradient workload: 'relaxed' --
    the field-free ground state by imaginary-time relaxation from seed-42
    orbitals; 'correlated' -- seed-42 Gaussian orbitals with a seeded random
    normalised CI vector, every natural orbital occupied."""
    from codyfortran_gb300 import init as I
    from codyfortran_gb300 import spec as S
    sp0 = S.helium_fedvr(100, 6, 8, laser=S.Laser())
    orbs = I.seeded_gaussian_orbitals(sp0, x, w, 42)
    if kind == "relaxed":
        st0 = I.pack_state(I.unary_coeffs(sp0), orbs)
        e0, st, rounds = eng_relax.relax(st0, 0.005, 10, 1e-12, 2000)
        return st, {"relaxed_energy": e0, "relax_rounds": rounds}
    rng = np.random.default_rng(42)
    c = rng.normal(size=sp0.n_coeffs) + 1j * rng.normal(size=sp0.n_coeffs)
    return I.pack_state(c / np.linalg.norm(c), orbs), {}


def run_adjoint(args):
    """--workload adjoint_helium: the pulse-gradient workload -- 1D helium
    (100 FEDVR elements x 6 points, 501 points), M = 8 restricted orbitals,
    --adjoint-samples field samples E_n ~ N(0, 0.01^2) from seed 99,
    dt = 0.05, Krylov order 12, checkpoints every 64 steps, objective
    1 - |<Psi_0|Psi_N>|^2.  Times one forward + backward evaluation (the
    gradient with respect to all samples) and compares central differences
    on a few random samples at h = 1e-5 and 1e-6."""
    from codyfortran_gb300 import build as B
    B.build()
    from codyfortran_gb300 import spec as S
    from codyfortran_gb300.engine import Engine
    nT, dt, K, chk = args.adjoint_samples, 0.05, 12, 64
    field = np.random.default_rng(99).normal(0.0, 0.01, size=4000)[:nT]
    mk = lambda laser: S.helium_fedvr(100, 6, 8, laser=laser)
    r = Engine(mk(S.Laser()))
    st, extra = adjoint_start_state(args.adjoint_state, r.x, r.w, r)
    r.close()
    e = Engine(mk(S.Laser(kind="sampled", samples=field, sample_dt=dt, sample_t0=0.0)), max_krylov=K)
    e.mc_adjoint_forward(st, field[:8], dt, K, chk)  # warm-up (allocations, module load)
    e.mc_adjoint_backward()
    t0 = time.perf_counter()
    J, ov, fin = e.mc_adjoint_forward(st, field, dt, K, chk)
    t1 = time.perf_counter()
    g = e.mc_adjoint_backward()
    t2 = time.perf_counter()
    idx = np.sort(np.random.default_rng(7).choice(nT, size=args.adjoint_fd, replace=False))
    rows, worst = [], {}
    gmax = float(np.max(np.abs(g)))
    fds = {}
    for h in (1e-5, 1e-6):
        worst[h] = 0.0
        for n in idx:
            f1, f2 = field.copy(), field.copy()
            f1[n] += h
            f2[n] -= h
            fd = (e.mc_adjoint_forward(st, f1, dt, K, chk)[0] - e.mc_adjoint_forward(st, f2, dt, K, chk)[0]) / (2 * h)
            rows.append((h, int(n), float(fd), float(g[n])))
            fds[(h, int(n))] = float(fd)
            worst[h] = max(worst[h], abs(fd - g[n]) / gmax)
    e.close()
    # a sample is inside the linear range of central differences when the two
    # step sizes agree to 1e-3; the relative error is judged on those samples
    per, worst_lin = [], 0.0
    for n in idx:
        a, b, gn = fds[(1e-5, int(n))], fds[(1e-6, int(n))], float(g[n])
        lin = abs(a - b) <= 1e-3 * max(abs(b), 1e-12)
        rel = abs(a - gn) / max(abs(gn), 1e-300)
        per.append({"sample": int(n), "adjoint": gn, "fd_1e-5": a, "fd_1e-6": b, "rel_err_1e-5": rel,
                    "fd_linear": lin})
        if lin:
            worst_lin = max(worst_lin, rel)
    line = {"metric": "MCTDHF pulse-gradient evaluations/s (forward + backward over all field samples)",
            "value": 1.0 / (t2 - t0), "unit": "gradients/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "complex128", "data": f"synthetic (seed-99 field samples; {args.adjoint_state} start state)",
            "config": dict({"workload": "adjoint_helium", "n_grid": 501, "n_orbitals": 8, "field_samples": nT,
                            "dt": dt, "krylov_order": K, "checkpoint": chk, "start_state": args.adjoint_state},
                           **extra),
            "forward_s": t1 - t0, "backward_s": t2 - t1, "objective": J, "survival": abs(ov) ** 2,
            "gradient_max_abs": gmax,
            "fd_check": {"samples": rows, "per_sample": per,
                         "worst_abs_diff_over_max_gradient": {str(k): v for k, v in worst.items()},
                         "samples_in_linear_range": sum(p["fd_linear"] for p in per),
                         "worst_rel_err_in_linear_range": worst_lin, "target": 1e-6}}
    print(json.dumps(line))
    return 0


def krylov_window(args, precision):
    """Lanczos re-orthogonalisation window: the reference's full loop for the
    FP64 form, the three-term recurrence (window 1) for the mixed forms unless
    --krylov-window says otherwise."""
    if args.krylov_window is not None:
        return args.krylov_window
    return 0 if precision == "fp64" else 1


def window_name(window):
    if window == 0:
        return "full (every basis vector)"
    if window == 1:
        return "three-term recurrence"
    return f"Gram-Schmidt against the last {window} basis vectors"


def run_batch(args):
    rank, world, local = dist_info()
    specs, cfg = workload(args.workload)
    precision = args.precision or "mixed_fx6"
    n = len(specs)
    window = krylov_window(args, precision)
    acc_steps = 0 if args.no_fp64_leg or precision == "fp64" else ACC_STEPS
    r = run_batch_leg(specs, cfg, precision, args.steps, args.warmup, profile=True, clock=True, acc_steps=acc_steps,
                      window=window)
    ms = barrier_max(r["ms"], world)
    value = world * n * args.steps / (ms / 1e3)
    # the same batch in the plain FP64 form with the reference's full Krylov
    # re-orthogonalisation (short timed region), and the deviation of the mixed
    # form from it after ACC_STEPS steps from the same states; with a Krylov
    # window also the FP64 form with that window, to separate the two gains
    fp64, fp64_win, accuracy = None, None, None
    fsteps = max(1, min(args.steps, 2))
    if acc_steps:
        f = run_batch_leg(specs, cfg, "fp64", fsteps, 1, profile=False, e2e=False, acc_steps=acc_steps)
        fp64 = n * fsteps / (f["ms"] / 1e3)
        if window:
            fw = run_batch_leg(specs, cfg, "fp64", fsteps, 1, profile=False, e2e=False, window=window)
            fp64_win = n * fsteps / (fw["ms"] / 1e3)
        dA = np.abs(r["acc_energy"] - f["acc_energy"])
        dE = dA / np.abs(f["acc_energy"])
        dS = dA / np.maximum(np.abs(f["acc_energy"]), 1.0)
        dN = np.abs(r["acc_norm"] - f["acc_norm"])
        worst = int(np.argmax(dE))
        accuracy = {"steps": acc_steps, "energy_rel_max": float(dE.max()), "energy_rel_median": float(np.median(dE)),
                    "energy_rel_p99": float(np.quantile(dE, 0.99)), "energy_abs_max": float(dA.max()),
                    "energy_rel_to_max_E_1Eh_max": float(dS.max()),
                    "fraction_energy_rel_within_target": float(np.mean(dE <= 1e-8)),
                    "fraction_energy_abs_within_target": float(np.mean(dA <= 1e-8)),
                    "worst": {"trajectory": worst, "energy_fp64": float(f["acc_energy"][worst]),
                              "n_orbitals": int(systems_of(r)[worst].nOS), "n_grid": int(systems_of(r)[worst].nG),
                              "n_determinants": int(systems_of(r)[worst].nC)},
                    "norm_abs_max": float(dN.max()), "norm_abs_median": float(np.median(dN)),
                    "target": 1e-8, "reference": "same batch, plain FP64 form on the GPU (parity-tested against "
                                                  "the CPU port to 1e-12)"}
    # roofline of the dominant kernel family, timed inside seconds of steps:
    # the sustained bf16 figure is its tensor denominator
    hbm, bf16, src = measured_peaks(sustained=True)
    dom, n_dom = r["dom"], max(r["n_dom"], 1)
    avg_s = r["ms_dom"] / n_dom / 1e3
    systems = r["systems"]
    roof = {"kernel": dom, "launches": r["n_dom"], "avg_launch_us": avg_s * 1e6, "peak_source": src, "traffic": None}
    if dom in ("pair_potentials", "correlation", "h2"):
        work = dense_flops(systems, dom) / n_dom
        roof.update(bound="tensor", achieved=work / avg_s / 1e12, peak=bf16, unit="TFLOP/s", work_per_launch=work)
        if precision in FX_BITS and dom in ("pair_potentials", "h2"):
            # what the tensor cores execute: every algorithmic product as slice products
            k = fx_grid_products(precision, systems)
            roof.update(slice_products_per_product=k, issued_tflops=k * roof["achieved"],
                        issued_frac=k * roof["achieved"] / bf16)
    elif dom == "lanczos":
        byts, flops = lanczos_work(systems, cfg["krylov"], window)
        byts /= n_dom
        roof.update(bound="hbm", achieved=byts / avg_s / 1e9, peak=hbm, unit="GB/s", work_per_launch=byts,
                    fp64_tflops=flops / n_dom / avg_s / 1e12)
    else:
        byts = sum(s.nS for s in systems) * 16.0 * 4
        roof.update(bound="hbm", achieved=byts / avg_s / 1e9, peak=hbm, unit="GB/s", work_per_launch=byts)
    roof["frac"] = roof["achieved"] / roof["peak"]
    prof = PROFILED_TRAFFIC.get((args.workload, precision, dom))
    if prof:
        roof.update(traffic=prof[0], traffic_unit="bytes per launch", traffic_source=prof[1])
    e2e = world * n / r["e2e_s"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPES[precision],
        "data": "synthetic (seeded Gaussian orbitals, random normalised CI vectors)",
        "config": {"workload": args.workload, "trajectories": n, "krylov_order": cfg["krylov"], "dt": cfg["dt"],
                   "precision": precision, "krylov_reorthogonalisation": window_name(window),
                   "parallelism": f"batch of {n} per GPU, replicas x{world}",
                   "tiles": "autotuned", "tile_table": r["tiles"],
                   "n_grid_range": [min(s.nG for s in systems), max(s.nG for s in systems)],
                   "n_determinants_range": [min(s.nC for s in systems), max(s.nC for s in systems)],
                   "l2": f"per-step working set {sum(s.nS for s in systems) * 16 * (cfg['krylov'] + 8) / 1e9:.1f} GB "
                         f"of states and Krylov vectors > L2 ({L2_BYTES / 1e6:.0f} MB): inputs larger than L2, no flush"},
        "fp64_gpu": {"value": fp64, "unit": UNIT, "ratio": (value / fp64) if fp64 else None,
                     "note": "same batch, plain FP64 form with full Krylov re-orthogonalisation (the reference's "
                             "algorithm), same GPU"},
        "fp64_gpu_same_krylov": None if fp64_win is None else {
            "value": fp64_win, "unit": UNIT, "ratio": value / fp64_win,
            "note": f"same batch, FP64 form with the timed leg's Krylov recurrence ({window_name(window)})"},
        "accuracy_vs_fp64": accuracy,
        "clocks": r["clocks"],
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": r["e2e_bytes"], "d2h_bytes_per_step": r["e2e_bytes"],
                "call": "cgpu_batch_upload + cgpu_batch_propagate(1 step) + cgpu_batch_download, pinned host "
                        "buffers (cgpu_host_alloc)"},
        "gpu_launches": int(r["launches"]),
        "kernels_per_step": r["kps"],
        "roofline": roof,
        "kernel_ms_per_step": {k: v[1] for k, v in r["fam_ms"].items()},
    }
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count()
        val, smp = oracle_parallel_traj_steps(specs, cfg, cores, n_sample=32, steps=1)
        line["cpu_baseline"] = {
            "value": val, "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(),
            "sample": f"{smp['timed_steps']} Strang steps over {smp['trajectories']} trajectories spread over "
                      f"{args.workload}, one trajectory per worker process and core (one OpenMP thread each): "
                      f"{cores} x steps / {smp['core_seconds']:.1f} summed core-seconds "
                      f"({smp['wall_seconds']:.1f} s wall)"}
    if rank == 0:
        print(json.dumps(line))
    return 0


def orbital_span_defect(a, b, nC, nG, n, w):
    """1 - |det <phi_a|phi_b>_w| over the stored orbitals of two states (0 when
    both orbital sets span the same space; invariant under rotations within it)."""
    fa = a[nC:nC + nG * n].reshape(n, nG)
    fb = b[nC:nC + nG * n].reshape(n, nG)
    return float(abs(1.0 - abs(np.linalg.det((fa.conj() * w) @ fb.T))))


def mixed_deviation(sp, cfg, precision, window, st, n_steps):
    """Per-step deviation of a mixed-precision trajectory from the FP64 form with
    the reference's Krylov loop, from the same state: |dE|/|E|, |d||C|||,
    |d<x>| and the orbital-span defect, each maximised over the steps."""
    from codyfortran_gb300.engine import Engine
    K, dt = cfg["krylov"], cfg["dt"]
    f = Engine(sp, precision="fp64", max_krylov=K, krylov_window=0)
    m = Engine(sp, precision=precision, max_krylov=K, krylov_window=window)
    f.upload(st)
    m.upload(st)
    t, rows = 0.0, []
    for _ in range(n_steps):
        f.propagate_resident(t, dt, 1, K, use_metric=True, use_graph=True)
        m.propagate_resident(t, dt, 1, K, use_metric=True, use_graph=True)
        t += dt
        of, om = f.observables(t), m.observables(t)
        rows.append((abs(om["energy"] - of["energy"]) / abs(of["energy"]), abs(om["norm"] - of["norm"]),
                     abs(om["dipole"] - of["dipole"]),
                     orbital_span_defect(m.download(), f.download(), f.nC, f.nG, f.nOS, f.w)))
    f.close()
    m.close()
    r = np.array(rows)
    return {"steps": n_steps, "energy_rel_max": float(r[:, 0].max()), "norm_abs_max": float(r[:, 1].max()),
            "dipole_abs_max": float(r[:, 2].max()), "orbital_span_defect_max": float(r[:, 3].max()),
            "energy_rel_last": float(r[-1, 0]), "target": 1e-8,
            "reference": "same state, plain FP64 form with the reference's Krylov loop on the GPU"}


def run_single(args):
    rank, world, local = dist_info()
    from codyfortran_gb300.engine import Engine, pinned_empty
    specs, cfg = workload(args.workload)
    sp = specs[0]
    precision = args.precision or "fp64"
    window = krylov_window(args, precision)
    e = Engine(sp, precision=precision, max_krylov=cfg["krylov"], krylov_window=window)
    st = initial_state(sp, e.x, e.w, cfg["seed"])
    dt, K = cfg["dt"], cfg["krylov"]
    e.upload(st)
    heuristic = e.tiles()
    rep = e.autotune()
    tiles = {"tiles": "autotuned", "source": rep["source"], "table": rep["tiles"], "heuristic": heuristic}
    e.upload(st)
    t = 0.0
    graph = not args.no_graph
    e.propagate_resident(t, dt, args.warmup, K, use_metric=True, use_graph=graph)
    t += args.warmup * dt
    e.synchronize()
    fam_ms = {}
    for fam in FAMILIES:
        e.profile_begin(fam)
        e.propagate_resident(t, dt, 1, K, use_metric=True, use_graph=graph)
        t += dt
        fam_ms[fam] = e.profile_end()
    dom = max(fam_ms, key=lambda k: fam_ms[k][1])
    e.profile_begin(dom)
    e.propagate_resident(t, dt, 1, K, use_metric=True, use_graph=graph)  # capture with the events, untimed
    t += dt
    e.launch_count(reset=True)
    with ClockSampler(0) as clk:
        ms = e.propagate_resident_timed(t, dt, args.steps, K, use_metric=True, use_graph=graph)
    n_dom, ms_dom = e.profile_end()
    launches = e.launch_count()
    t += args.steps * dt
    ms = barrier_max(ms, world)
    value = world * args.steps / (ms / 1e3)
    host = pinned_empty(e.nS)
    host[:] = e.download()
    n_e2e = max(1, min(args.steps, 20))
    # untimed: the step graph is re-captured without the profiling events
    e.propagate_split2(host, t, t + dt, krylov_dim=K, use_metric=True, out=host)
    t += dt
    te0 = time.perf_counter()
    for _ in range(n_e2e):
        e.propagate_split2(host, t, t + dt, krylov_dim=K, use_metric=True, out=host)
        t += dt
    te = barrier_max(time.perf_counter() - te0, world)
    e2e = world * n_e2e / te
    hbm, bf16, src = measured_peaks(sustained=True)
    nG, P, Q, nC = e.nG, e.nOS * (e.nOS + 1) // 2, e.nOS * e.nOS, e.nC
    avg_s = (ms_dom / max(n_dom, 1)) / 1e3
    if dom == "pair_potentials":
        work, bound = 2.0 * nG * nG * 2 * P, "tensor"
    elif dom in ("correlation", "h2"):
        work, bound = 8.0 * nG * Q * Q, "tensor"
    elif dom == "lanczos":
        work, bound = lanczos_work([e], K, window)[0] / max(n_dom, 1), "hbm"
    else:
        work, bound = 16.0 * e.nS * 4, "hbm"
    if bound == "tensor":
        achieved, peak, unit = work / avg_s / 1e12, bf16, "TFLOP/s"
    else:
        achieved, peak, unit = work / avg_s / 1e9, hbm, "GB/s"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPES[precision],
        "data": "synthetic (seeded Gaussian orbitals, random normalised CI vector)",
        "config": {"workload": args.workload, "n_grid": nG, "n_orbitals": e.nOS, "n_determinants": nC,
                   "krylov_order": K, "dt": dt, "precision": precision,
                   "krylov_reorthogonalisation": window_name(window), "parallelism": f"replicas x{world}",
                   "tiles": "autotuned", "tile_table": tiles,
                   "l2": "inputs larger than L2, no flush"},
        "clocks": clk.summary(),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": e.nS * 16, "d2h_bytes_per_step": e.nS * 16,
                "steps": n_e2e, "call": "cgpu_propagate_split2 (host state in/out, pinned host buffer)"},
        "gpu_launches": int(launches),
        "roofline": {"kernel": dom, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
                     "frac": achieved / peak, "peak_source": src, "traffic": None,
                     "launches": n_dom, "avg_launch_us": avg_s * 1e6, "work_per_launch": work},
        "kernel_ms_per_step": {k: v[1] for k, v in fam_ms.items()},
    }
    if rank == 0 and precision != "fp64" and not args.no_fp64_leg:
        line["accuracy_vs_fp64"] = mixed_deviation(sp, cfg, precision, window, st, ACC_STEPS_SINGLE)
    if rank == 0 and not args.no_cpu_baseline:
        steps_cpu, el, used = oracle_traj_steps(specs, cfg, os.cpu_count(), args.cpu_budget)
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
    ap.add_argument("--workload", default="batch512",
                    choices=["batch512", "trimer_large", "helium_small", "adjoint_helium"])
    ap.add_argument("--adjoint-samples", type=int, default=4000, help="adjoint_helium: field samples (steps)")
    ap.add_argument("--adjoint-state", default="correlated", choices=["correlated", "relaxed"],
                    help="adjoint_helium: start and reference state")
    ap.add_argument("--adjoint-fd", type=int, default=4, help="adjoint_helium: samples checked by central differences")
    ap.add_argument("--precision", default=None, choices=list(DTYPES))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-leg", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=25.0)
    ap.add_argument("--no-graph", action="store_true", help="launch kernels one by one instead of a step graph")
    ap.add_argument("--accuracy-horizon", type=int, default=0,
                    help="instead of timing: per-step deviation of the mixed form from FP64 over this many steps")
    ap.add_argument("--accuracy-trajectories", type=int, default=32)
    ap.add_argument("--accuracy-every", type=int, default=10)
    ap.add_argument("--krylov-window", type=int, default=None,
                    help="0: Gram-Schmidt against all Krylov vectors; 1: three-term recurrence; k > 1: against the "
                         "last k (default 0 for fp64, 1 otherwise)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.accuracy_horizon:
        return run_accuracy_horizon(args)
    if args.workload == "adjoint_helium":
        return run_adjoint(args)
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from codyfortran_gb300 import build as B
    B.build()
    if world > 1:
        from codyfortran_gb300.engine import select_device
        select_device(local)  # one replica per GPU
    if args.workload == "batch512":
        return run_batch(args)
    return run_single(args)


if __name__ == "__main__":
    sys.exit(main())
