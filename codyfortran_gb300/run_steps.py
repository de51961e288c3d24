"""Advance a benchmark workload by a few steps on the GPU (for profilers).

    python -m codyfortran_gb300.run_steps --workload batch512 --precision mixed_fx --steps 1 [--trajectories N]

Builds the workload (the 512-trajectory batch, or a prefix of it, or the
trimer), uploads seeded initial states and propagates --steps Strang steps
(the first one captures the step graph).  Prints the number of kernels
launched before the first step, so that a profiler can skip the set-up.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    from codyfortran_gb300 import init as I
    from codyfortran_gb300 import spec as S
    from codyfortran_gb300.engine import Batch, Engine

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="batch512", choices=["batch512", "trimer_large"])
    ap.add_argument("--precision", default="mixed_fx6", choices=["fp64", "mixed", "mixed6", "mixed_fx", "mixed_fx6"])
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--trajectories", type=int, default=512)
    ap.add_argument("--krylov-window", type=int, default=None,
                    help="Lanczos re-orthogonalisation window (default: 0 for fp64, 1 = three-term recurrence for mixed forms)")
    args = ap.parse_args()
    window = args.krylov_window if args.krylov_window is not None else (0 if args.precision == "fp64" else 1)

    def state(sp, x, w, seed):
        rng = np.random.default_rng(seed)
        orbs = I.seeded_gaussian_orbitals(sp, x, w, seed)
        c = rng.normal(size=sp.n_coeffs) + 1j * rng.normal(size=sp.n_coeffs)
        return I.pack_state(c / np.linalg.norm(c), orbs)

    if args.workload == "batch512":
        specs = S.batch_trajectory_specs(512, 1234)[: args.trajectories]
        b = Batch(specs, args.precision, max_krylov=12, krylov_window=window)
        b.upload([state(sp, s.x, s.w, 1234 + k) for k, (sp, s) in enumerate(zip(specs, b.systems))])
        print("set-up launches", b.launch_count(), flush=True)
        ms = b.propagate(0.0, 0.02, args.steps, 12)
        print(f"steps {args.steps} device ms {ms:.3f} kernels/step {b.kernels_per_step()}")
        b.close()
    else:
        sp = S.cfg_trimer_large()
        e = Engine(sp, args.precision, max_krylov=16, krylov_window=window)
        e.upload(state(sp, e.x, e.w, 7))
        print("set-up launches", e.launch_count(), flush=True)
        ms = e.propagate_resident_timed(0.0, 0.02, args.steps, 16, use_metric=True, use_graph=True)
        print(f"steps {args.steps} device ms {ms:.3f}")
        e.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
