"""Pins the CPU oracle against the reference's own golden values and known answers.

Each test restates one check of the reference test suite (file:line recorded in
tests/golden/he1d_golden.json) on the oracle.
"""
import numpy as np
import pytest

from oracle import Oracle, gll, eig_herm, eig_sym
from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S


def _gold(golden, key, i=0):
    return golden[key]["checks"][i]["golden"]


def test_gll_closed_forms():
    x, w = gll(3)
    np.testing.assert_allclose(x, [-1, 0, 1], atol=1e-15)
    np.testing.assert_allclose(w, [1 / 3, 4 / 3, 1 / 3], atol=1e-15)
    x, w = gll(4)
    np.testing.assert_allclose(x, [-1, -1 / np.sqrt(5), 1 / np.sqrt(5), 1], atol=1e-15)
    np.testing.assert_allclose(w, [1 / 6, 5 / 6, 5 / 6, 1 / 6], atol=1e-15)
    x, w = gll(5)
    np.testing.assert_allclose(x, [-1, -np.sqrt(3 / 7), 0, np.sqrt(3 / 7), 1], atol=1e-15)
    for n in (6, 8, 12, 21):
        x, w = gll(n, -0.5, 0.5)
        for k in range(2 * n - 2):  # exact for polynomials of degree <= 2n-3
            exact = (0.5 ** (k + 1) - (-0.5) ** (k + 1)) / (k + 1)
            assert abs(np.sum(w * x ** k) - exact) < 1e-14


def test_fedvr_derivative_pin():
    """test/componentTests/Utils/T_Utils_DerivativeFedvr.f90:20-126: 10 elements x 21
    points on [0,20], lower endpoint excluded, f = r exp(-2r); rel. err < 1e-8."""
    sp = S.SystemSpec(grid_kind="fedvr", xmin=0.0, xmax=20.0, n_elements=10, n_locals=21, xmin_excluded=True,
                      n_bodies=(1,), n_orbs=(1,), has_interaction=False)
    o = Oracle(sp)
    r, lam = o.x, 2.0
    f = r * np.exp(-lam * r)
    d2 = o.fedvr_derivative(f, 2)
    e2 = (-2 * lam + lam ** 2 * r) * np.exp(-lam * r)
    d1 = o.fedvr_derivative(f, 1)
    e1 = (1 - lam * r) * np.exp(-lam * r)
    assert np.max(np.abs(d2 - e2)) / np.max(np.abs(e2)) < 1e-8
    assert np.max(np.abs(d1 - e1)) / np.max(np.abs(e1)) < 1e-8


def test_eigensolvers_match_numpy():
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 16):
        A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        A = A + A.conj().T
        ev, U = eig_herm(A)
        np.testing.assert_allclose(ev, np.linalg.eigvalsh(A), atol=1e-12)
        np.testing.assert_allclose(U @ np.diag(ev) @ U.conj().T, A, atol=1e-12)
        B = rng.normal(size=(n, n))
        B = B + B.T
        ev, U = eig_sym(B)
        np.testing.assert_allclose(ev, np.linalg.eigvalsh(B), atol=1e-12)


def test_tdci_exact_diag_pin(golden):
    """He1d_02 (T_He1d_02_ExactDiagTdci.f90:74): TDCI with 21+21 grid-point orbitals
    spans the full two-electron grid space; its ground state is the exact one."""
    sp = S.he1d_findiff(n_orbs=(21, 21))
    sp.method = "tdci"
    o = Oracle(sp)
    o.tdci_set_orbitals(I.grid_point_orbitals(sp, o.w))
    n = o.nC
    H = np.zeros((n, n), dtype=complex)
    for j in range(n):
        e = np.zeros(n, dtype=complex)
        e[j] = 1.0
        H[:, j] = 1j * o.time_derivative(e, 0.0, "tdci")
    assert np.abs(H - H.conj().T).max() < 1e-12
    e0 = np.linalg.eigvalsh(H)[0]
    assert abs(e0 - _gold(golden, "he1d_02_tdci_exact_diag")) < 1e-12
    assert abs(e0 - _gold(golden, "he1d_01_exact_diag")) < 1e-12


def _relax(n_orbs, restricted):
    sp = S.he1d_findiff(n_orbs=n_orbs, restricted=restricted)
    o = Oracle(sp)
    orbs = I.orthonormalize_state_orbitals(sp, I.harmonic_orbitals(sp, o.x), o.w)
    st = I.pack_state(I.unary_coeffs(sp), orbs)
    e, st, _ = o.relax(st, 0.01, 10, 1e-12)
    return o, e, st


def test_hartree_fock_relax_pin(golden):
    """He1d_03 (T_He1d_03_ImagTimePropagationTdhx.f90:107): one orbital per spin
    makes the MCTDHF equations the TDHF ones."""
    _, e, _ = _relax((1, 1), False)
    assert abs(e - _gold(golden, "he1d_03_tdhf_imag")) < 1e-8


@pytest.mark.parametrize("restricted,key", [(False, "he1d_04_mctdhf_imag"), (True, "he1d_07_mctdhf_imag_restricted")])
def test_mctdhf_relax_pin(golden, restricted, key):
    _, e, _ = _relax((4, 4), restricted)
    assert abs(e - _gold(golden, key)) < 1e-8


@pytest.mark.parametrize("krylov", [0, 24])
def test_realtime_split_pin(golden, krylov):
    """He1d_05 (RK4+RK4, :122) and He1d_06 (SIL(24, 1e-12, 8)+RK4, :130-140):
    t in [0, 1e-3], dt = 1e-5.  The golden drift E(T) - E(0) is reproduced to
    1e-10 and the final energy to the reference tolerance."""
    o, e_relaxed, st = _relax((4, 4), False)
    e0 = o.energy(st, 0.0)
    n0 = np.linalg.norm(st)
    t, dt = 0.0, 0.00002 / 2
    while t < 0.001:
        for _ in range(2):
            st = o.propagate_split2(st, t, t + dt, krylov_dim=krylov, tol=1e-12, max_restarts=8)
            t = t + dt
    e = o.energy(st, t)
    gold_final = _gold(golden, "he1d_05_mctdhf_split_rk4")
    gold_drift = gold_final - _gold(golden, "he1d_04_mctdhf_imag")
    assert abs((e - e0) - gold_drift) < 1e-10
    assert abs(e - gold_final) < 1e-7
    assert abs(e - e0) < 1e-6
    if krylov:
        assert abs(np.linalg.norm(st) - n0) < 1e-10


def test_configlist_sizes_large():
    """N=6 fermions in 16 orbitals: C(16,6) = 8008 determinants, 6*11 = 66 singles
    and C(6,2)*C(12,2) = 990 doubles per determinant."""
    sp = S.SystemSpec(grid_kind="const", xmin=-1, xmax=1, n_points=12, n_bodies=(6,), n_orbs=(16,), masses=(1.0,),
                      has_interaction=False)
    o = Oracle(sp)
    s = o.tables(0, 0)
    d = o.tables(0, 1)
    assert o.nC == 8008
    assert (s["n_connected"] == 66).all() and (d["n_connected"] == 990).all()
    assert s["codes"][0] == 0b111111 and s["codes"][-1] == 0b1111110000000000
