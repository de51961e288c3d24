"""System specification: the JSON configuration tree of one MCTDHX/TDCI run.

The fields mirror the reference's configuration keys that select and
parameterise the hot path:

* ``grid.linear.{xmin,xmax}`` with ``const.nPoints`` (src/Grid/Linear/S_Grid_Linear.f90:29-30,
  src/Grid/Linear/Const/S_Grid_Linear_Const.f90:23) or FEDVR elements
  (src/Utils/M_Utils_Fedvr.f90:76-149; ``n_locals`` = points per element = order + 1).
* ``sysKinetic.linear.laplacian.bodyMass`` (finite differences on ``const`` grids,
  the 1D FEDVR operator on ``fedvr`` grids).
* ``sysPotential.linear.softYukawa.{position,charge,softening1,softening2,dampening}``
  (src/SysPotential/Linear/SoftYukawa/S_SysPotential_Linear_SoftYukawa.f90:33-43).
* ``sysInteraction.linear.softYukawa.{strength,softening1,softening2,dampening}``
  (src/SysInteraction/Linear/SoftYukawa/S_SysInteraction_Linear_SoftYukawa.f90:33-36).
* a 1D length-gauge laser, E(t) x, with the sin^2 pulse of
  src/SysPotential/Ylm/CoulombLaser/S_SysPotential_Ylm_CoulombLaser.f90:60-83, or a
  piecewise-constant sampled field for pulse optimisation.
* ``method.mb.{nBodyTypes,nBodies,bodyStatistics}``, ``method.mb.orbBased.{nOrbs,
  regularizationParameter}`` and ``orbs.restrictedQ``
  (src/Method/Mb/S_Method_Mb.f90:51-61, src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90:56-79).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np


@dataclasses.dataclass
class Nucleus:
    position: float
    charge: float
    softening1: float = 1.0
    softening2: float = 0.0
    dampening: float = 0.0


@dataclasses.dataclass
class Laser:
    """kind: 'none' | 'sin2' (analytic pulse) | 'sampled' (E_n on [t0 + n dt, t0 + (n+1) dt))."""
    kind: str = "none"
    E0: float = 0.0
    omega: float = 0.0
    n_cycles: float = 0.0
    cep: float = 0.0
    t_start: float = 0.0
    samples: Optional[np.ndarray] = None
    sample_dt: float = 1.0
    sample_t0: float = 0.0

    def amplitude(self, t: float) -> float:
        if self.kind == "sin2":
            if self.omega <= 0.0:
                return 0.0
            duration = 2.0 * math.pi * self.n_cycles / self.omega
            tr = t - self.t_start
            if tr < 0.0 or tr > duration:
                return 0.0
            env = math.sin(math.pi * tr / duration) ** 2
            return self.E0 * env * math.cos(self.omega * (tr - 0.5 * duration) + self.cep)
        if self.kind == "sampled":
            n = int(math.floor((t - self.sample_t0) / self.sample_dt + 1e-9))
            if n < 0 or n >= len(self.samples):
                return 0.0
            return float(self.samples[n])
        return 0.0


@dataclasses.dataclass
class SystemSpec:
    # grid
    grid_kind: str = "const"          # 'const' (finite differences) | 'fedvr'
    xmin: float = -10.0
    xmax: float = 10.0
    n_points: int = 100               # const grid
    n_elements: int = 10              # fedvr
    n_locals: int = 9                 # fedvr points per element (order + 1)
    xmin_excluded: bool = False
    xmax_excluded: bool = False
    # bodies / orbitals
    n_bodies: Sequence[int] = (1,)
    n_orbs: Sequence[int] = (1,)
    masses: Sequence[float] = (1.0,)
    stats: str = "f"
    restricted: bool = False
    reg_eps: float = 1e-10
    # operators
    nuclei: List[Nucleus] = dataclasses.field(default_factory=list)
    has_interaction: bool = True
    int_strength: float = 1.0
    int_s1: float = 1.0
    int_s2: float = 0.0
    int_damp: float = 0.0
    int_kind: str = "dense"           # 'toeplitz' (uniform grid, K(|i-j| dx)) | 'dense' (K(|x_i-x_j|))
    laser: Laser = dataclasses.field(default_factory=Laser)
    method: str = "mctdhx"            # 'mctdhx' | 'tdci'

    @property
    def n_bt(self) -> int:
        return len(self.n_bodies)

    @property
    def n_grid(self) -> int:
        if self.grid_kind == "const":
            return self.n_points
        n = self.n_elements * (self.n_locals - 1) + 1
        return n - int(self.xmin_excluded) - int(self.xmax_excluded)

    @property
    def n_orbs_sum(self) -> int:
        return int(sum(self.n_orbs))

    @property
    def n_orbs_in_state(self) -> int:
        return int(self.n_orbs[0]) if self.restricted else self.n_orbs_sum

    @property
    def n_coeffs(self) -> int:
        n = 1
        for m, k in zip(self.n_orbs, self.n_bodies):
            n *= math.comb(int(m), int(k))
        return n

    @property
    def n_state(self) -> int:
        if self.method == "tdci":
            return self.n_coeffs
        return self.n_coeffs + self.n_grid * self.n_orbs_in_state


# ---------------------------------------------------------------------------
# Named workloads.  Sizes and parameters follow the benchmark definitions:
# soft-Coulomb 1D models on FEDVR grids with a length-gauge sin^2 pulse.
# ---------------------------------------------------------------------------

def he1d_findiff(n_orbs=(4, 4), restricted=False) -> SystemSpec:
    """The reference's He1d golden chain: 21-point finite-difference grid on
    [-20,20], V = -2/(|x|+1), W = 1/(|x-x'|+1)
    (test/simulationTests/He1d/T_He1d_04_ImagTimePropagationMctdhx.json)."""
    return SystemSpec(
        grid_kind="const", xmin=-20.0, xmax=20.0, n_points=21,
        n_bodies=(1, 1), n_orbs=tuple(n_orbs), masses=(1.0, 1.0), stats="ff", restricted=restricted,
        nuclei=[Nucleus(0.0, 2.0, 0.0, 1.0, 0.0)],
        has_interaction=True, int_strength=1.0, int_s1=0.0, int_s2=1.0, int_damp=0.0, int_kind="toeplitz",
    )


def helium_fedvr(n_elements=100, n_locals=6, n_orbs=4, laser=None, restricted=True) -> SystemSpec:
    """1D helium: V = -2/sqrt(x^2+1), W = 1/sqrt((x-x')^2+1), FEDVR grid on
    [-100,100], two spin body types with one electron each."""
    return SystemSpec(
        grid_kind="fedvr", xmin=-100.0, xmax=100.0, n_elements=n_elements, n_locals=n_locals,
        n_bodies=(1, 1), n_orbs=(n_orbs, n_orbs), masses=(1.0, 1.0), stats="ff", restricted=restricted,
        nuclei=[Nucleus(0.0, 2.0, 1.0, 0.0, 0.0)],
        has_interaction=True, int_strength=1.0, int_s1=1.0, int_s2=0.0, int_damp=0.0, int_kind="dense",
        laser=laser or Laser(),
    )


def sin2_pulse(E0: float, omega: float = 0.057, n_cycles: float = 4.0, cep: float = 0.0) -> Laser:
    return Laser(kind="sin2", E0=E0, omega=omega, n_cycles=n_cycles, cep=cep, t_start=0.0)


def cfg_helium_small() -> SystemSpec:
    """Plain MCTDHF 1D helium: 100 elements x 6 GLL points on [-100,100]
    (501 points), N=2 in M=4 spatial orbitals (restricted), E0 = 0.0534 au."""
    return helium_fedvr(100, 6, 4, laser=sin2_pulse(0.0534))


def cfg_trimer_large() -> SystemSpec:
    """Plain MCTDHF at scale: three soft-Coulomb nuclei Z=2 at x=-4,0,4,
    400 elements x 8 points on [-400,400] (2801 points), N=6 fermions in 16
    spin-orbitals (8008 determinants), E0 = 0.0755 au."""
    return SystemSpec(
        grid_kind="fedvr", xmin=-400.0, xmax=400.0, n_elements=400, n_locals=8,
        n_bodies=(6,), n_orbs=(16,), masses=(1.0,), stats="f", restricted=False,
        nuclei=[Nucleus(-4.0, 2.0, 1.0, 0.0, 0.0), Nucleus(0.0, 2.0, 1.0, 0.0, 0.0), Nucleus(4.0, 2.0, 1.0, 0.0, 0.0)],
        has_interaction=True, int_strength=1.0, int_s1=1.0, int_s2=0.0, int_damp=0.0, int_kind="dense",
        laser=sin2_pulse(0.0755),
    )


def cfg_adjoint_helium(seed: int = 99, n_samples: int = 4000, dt: float = 0.05) -> SystemSpec:
    """Pulse optimisation system: 1D helium (501 points), M=8 restricted,
    field sampled at n_samples points, E_n ~ N(0, 0.01^2)."""
    rng = np.random.default_rng(seed)
    samples = rng.normal(0.0, 0.01, size=n_samples)
    return helium_fedvr(100, 6, 8, laser=Laser(kind="sampled", samples=samples, sample_dt=dt, sample_t0=0.0))


def batch_trajectory_specs(n_traj: int = 512, seed: int = 1234, omega: float = 0.057):
    """Uneven batch of independent trajectories: N in {2,4} as two spin body
    types of N/2 electrons (restricted), M uniform in 4..12 spatial orbitals,
    FEDVR element counts uniform in 100..400 with 6 points each (domain
    [-nE, nE]), intensity log-uniform in 1e13..1e15 W/cm^2, CEP uniform in [0, 2 pi)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_traj):
        n = int(rng.choice([2, 4]))
        m = int(rng.integers(4, 13))
        ne = int(rng.integers(100, 401))
        inten = 10.0 ** rng.uniform(13.0, 15.0)
        cep = float(rng.uniform(0.0, 2.0 * math.pi))
        E0 = math.sqrt(inten / 3.509e16)
        spec = helium_fedvr(ne, 6, m, laser=sin2_pulse(E0, omega, 4.0, cep))
        spec.xmin, spec.xmax = -float(ne), float(ne)
        spec.n_bodies = (n // 2, n // 2)
        out.append(spec)
    return out
