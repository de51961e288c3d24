"""Initial orbitals and coefficients (OrbsInit / CoeffsInit extensions).

* ``harmonic_orbitals``: src/OrbsInit/Linear/Harmonic/S_OrbsInit_Linear_Harmonic.f90:52-80.
  The reference evaluates exp(-xi^2/2) * SfGslLib_Hermite(xi, n), and
  SfGslLib_Hermite (src/Utils/M_Utils_SfGslLib.f90:124-146) already carries an
  exp(-xi^2/2) factor, so the orbital is H_n(xi) exp(-xi^2) (unnormalised).
* ``seeded_gaussian_orbitals``: a seeded initialiser (the reference's random
  module seeds from the clock, src/Utils/M_Utils_Random.f90:13-30).  Complex
  Gaussian-envelope orbitals exp(-(x-x0)^2 / (2 sigma^2)) * (a + i b) with x0,
  sigma, a, b drawn from numpy's PCG64 generator, then orthonormalised by two
  modified Gram-Schmidt sweeps in the grid metric.
* ``unary_coeffs``: src/CoeffsInit/Unary (c_1 = 1).
* ``grid_point_orbitals``: src/OrbsInit/GridPoint/S_OrbsInit_GridPoint.f90:30-52.
"""
from __future__ import annotations

import numpy as np

from .spec import SystemSpec


def _hermite_phys(n: int, x: np.ndarray) -> np.ndarray:
    h0 = np.ones_like(x)
    if n == 0:
        return h0
    h1 = 2.0 * x
    for k in range(1, n):
        h0, h1 = h1, 2.0 * x * h1 - 2.0 * k * h0
    return h1


def harmonic_orbitals(spec: SystemSpec, x: np.ndarray, position: float = 0.0, omega: float = 1.0) -> np.ndarray:
    """(nG, nOS) complex orbitals; restricted runs store body type 1 only."""
    n_bt = 1 if spec.restricted else spec.n_bt
    cols = []
    a = 1.0 / np.sqrt(omega)
    xi = (x - position) / a
    for bt in range(n_bt):
        for ind in range(spec.n_orbs[bt]):
            cols.append(np.exp(-0.5 * xi ** 2) * _hermite_phys(ind, xi) * np.exp(-0.5 * xi ** 2))
    return np.array(cols, dtype=np.complex128).T.copy(order="F")


def grid_point_orbitals(spec: SystemSpec, w: np.ndarray) -> np.ndarray:
    n_bt = 1 if spec.restricted else spec.n_bt
    nG = len(w)
    cols = []
    for bt in range(n_bt):
        for ind in range(spec.n_orbs[bt]):
            o = np.zeros(nG, dtype=np.complex128)
            o[ind] = 1.0
            o /= np.sqrt(w[ind])
            cols.append(o)
    return np.array(cols).T.copy(order="F")


def mgs_orthonormalize(orbs: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Two modified Gram-Schmidt sweeps in the weighted metric (src/Grid/S_Grid.f90:120-151)."""
    f = np.array(orbs, dtype=np.complex128, order="F", copy=True)
    for i in range(f.shape[1]):
        for _ in range(2):
            for j in range(i):
                ov = np.sum(np.conj(f[:, j]) * f[:, i] * w)
                f[:, i] -= f[:, j] * ov
        nrm = np.sum(np.abs(f[:, i]) ** 2 * w).real
        if not nrm > 0.0:
            raise RuntimeError("Grid Orthonormalize: vector with non-positive norm")
        f[:, i] /= np.sqrt(nrm)
    return f


def orthonormalize_state_orbitals(spec: SystemSpec, orbs: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Orbs_Orthonormalize (src/Orbs/S_Orbs.f90:145-173): one block when restricted, else per body type."""
    if spec.restricted:
        return mgs_orthonormalize(orbs, w)
    out = np.array(orbs, dtype=np.complex128, order="F", copy=True)
    s = 0
    for m in spec.n_orbs:
        out[:, s:s + m] = mgs_orthonormalize(out[:, s:s + m], w)
        s += m
    return out


def seeded_gaussian_orbitals(spec: SystemSpec, x: np.ndarray, w: np.ndarray, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    nOS = spec.n_orbs_in_state
    span = 0.05 * (x[-1] - x[0])
    cols = []
    for _ in range(nOS):
        x0 = rng.uniform(-0.25 * span, 0.25 * span)
        sigma = rng.uniform(0.5, 2.5)
        a, b = rng.normal(size=2)
        cols.append(np.exp(-((x - x0) ** 2) / (2.0 * sigma ** 2)) * (a + 1j * b))
    orbs = np.array(cols, dtype=np.complex128).T.copy(order="F")
    return orthonormalize_state_orbitals(spec, orbs, w)


def unary_coeffs(spec: SystemSpec) -> np.ndarray:
    c = np.zeros(spec.n_coeffs, dtype=np.complex128)
    c[0] = 1.0
    return c


def pack_state(coeffs: np.ndarray, orbs: np.ndarray) -> np.ndarray:
    """Method_state = [C(nC) | orbs(nG, nOS) column-major]
    (src/Method/Mb/OrbBased/Mctdhx/S_Method_Mb_OrbBased_Mctdhx.f90:229-249)."""
    return np.concatenate([np.asarray(coeffs, dtype=np.complex128),
                           np.asarray(orbs, dtype=np.complex128).ravel(order="F")])


def unpack_state(state: np.ndarray, n_coeffs: int, n_grid: int):
    c = state[:n_coeffs]
    orbs = state[n_coeffs:].reshape(-1, n_grid).T
    return c, orbs
