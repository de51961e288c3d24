"""Host-side helpers of the parity tests (numpy, test infrastructure only).

mctdhf_overlap: <Psi_a|Psi_b> of two MCTDHF states with different orbital
sets, sum_{I,J} conj(Ca_I) Cb_J <Phi^a_I|Phi^b_J>, where the determinant
overlap is the product over body types of det(S_bt[occ(I), occ(J)]) and
S_bt = phi^a_bt^H W phi^b_bt is the grid-weighted orbital overlap of the body
type (restricted runs: the one stored spatial block for every body type).
Configurations are the reference's: per body type the k-subsets of the
orbitals in lexicographic order (bit i-1 of the code = orbital i), and the
global index mixed-radix over the body types with body type 1 fastest
(src/Coeffs/Generic/S_Coeffs_Generic.f90:625-639).

one_body_density: n(x) = sum_{ij} rho1(i,j)-weighted orbital products on the
grid, the gauge-invariant density of a state (independent of rotations among
the orbitals, and only weighted by occupation in the weakly occupied ones).
"""
from __future__ import annotations

import itertools

import numpy as np


def _configs(n_orbs, n_bodies):
    return [c for c in itertools.combinations(range(n_orbs), n_bodies)]


def mctdhf_overlap(spec, nG, w, sa, sb):
    n_bt = spec.n_bt
    nC = spec.n_coeffs
    nOS = spec.n_orbs_in_state
    fa = sa[nC:nC + nG * nOS].reshape(nOS, nG).T
    fb = sb[nC:nC + nG * nOS].reshape(nOS, nG).T
    Ca, Cb = sa[:nC], sb[:nC]
    S, occs, start = [], [], 0
    for bt in range(n_bt):
        m = spec.n_orbs[bt]
        s0 = 0 if spec.restricted else start
        S.append((fa[:, s0:s0 + m].conj() * w[:, None]).T @ fb[:, s0:s0 + m])
        occs.append(_configs(m, spec.n_bodies[bt]))
        start += m
    # per body type, the determinant-overlap matrix over its configurations
    D = []
    for bt in range(n_bt):
        oc = occs[bt]
        D.append(np.array([[np.linalg.det(S[bt][np.ix_(p, q)]) for q in oc] for p in oc]))
    # the global overlap matrix is the Kronecker product (body type 1 fastest)
    G = D[0]
    for bt in range(1, n_bt):
        G = np.kron(D[bt], G)
    return complex(Ca.conj() @ (G @ Cb))


def one_body_density(nG, nC, nOS, st, rdm1_spatial):
    f = st[nC:nC + nG * nOS].reshape(nOS, nG).T
    return np.real(np.einsum("xi,ij,xj->x", f, rdm1_spatial.T, f.conj()))


def grid_wavefunction_2e(spec, nG, st):
    """Psi(x1, x2) on the grid for two body types of one particle each
    (restricted: the one stored orbital set for both): Phi C Phi^T with
    C[i1, i2] = coefficient i1 + M i2 (body type 1 fastest)."""
    assert spec.n_bt == 2 and tuple(spec.n_bodies) == (1, 1)
    m1, m2 = spec.n_orbs[0], spec.n_orbs[1]
    nC = m1 * m2
    nOS = spec.n_orbs_in_state
    f = st[nC:nC + nG * nOS].reshape(nOS, nG).T
    f1 = f[:, :m1]
    f2 = f[:, :m2] if spec.restricted else f[:, m1:m1 + m2]
    C = st[:nC].reshape(m2, m1).T
    return f1 @ C @ f2.T


def wavefunction_distance(spec, nG, w, sa, sb):
    """||Psi_a - Psi_b|| / ||Psi_b|| in the grid metric (two one-particle body types)."""
    A = grid_wavefunction_2e(spec, nG, sa)
    B = grid_wavefunction_2e(spec, nG, sb)
    W = np.outer(w, w)
    return float(np.sqrt(np.sum(W * np.abs(A - B) ** 2) / np.sum(W * np.abs(B) ** 2)))
