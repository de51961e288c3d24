"""Parity of the GB300 engine (through the C ABI) with the CPU oracle.

FP64 form: relative error <= 1e-12 (||gpu - oracle|| / ||oracle||) on the same
seeded inputs; configuration tables bit-exact; golden values of the
reference's He1d tests reproduced on the GPU.
"""
import numpy as np
import pytest

from oracle import Oracle
from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b.ravel())
    return np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0)


def _single_bt():
    return S.SystemSpec(
        grid_kind="fedvr", xmin=-16.0, xmax=16.0, n_elements=16, n_locals=8,
        n_bodies=(3,), n_orbs=(6,), masses=(1.0,), stats="f", restricted=False,
        nuclei=[S.Nucleus(-2.0, 1.5, 1.0, 0.0, 0.0), S.Nucleus(2.0, 1.5, 1.0, 0.0, 0.1)],
        int_s1=1.0, int_kind="dense", laser=S.sin2_pulse(0.05, omega=0.3, n_cycles=2.0, cep=0.4))


def _helium_r():
    sp = S.helium_fedvr(20, 6, 4, laser=S.sin2_pulse(0.0534, omega=0.2, n_cycles=2.0))
    sp.xmin, sp.xmax = -20.0, 20.0
    return sp


def _two_electron_per_spin():
    sp = S.helium_fedvr(12, 6, 5, laser=S.sin2_pulse(0.03, omega=0.25, n_cycles=2.0, cep=1.0))
    sp.xmin, sp.xmax = -12.0, 12.0
    sp.n_bodies = (2, 2)
    return sp


SYSTEMS = {
    "he1d_unrestricted": lambda: S.he1d_findiff((4, 4), False),
    "he1d_restricted": lambda: S.he1d_findiff((3, 3), True),
    "helium_fedvr_restricted": _helium_r,
    "single_body_type": _single_bt,
    "two_per_spin_restricted": _two_electron_per_spin,
}


def _state(sp, o, seed):
    rng = np.random.default_rng(seed)
    orbs = I.seeded_gaussian_orbitals(sp, o.x, o.w, seed)
    c = rng.normal(size=o.nC) + 1j * rng.normal(size=o.nC)
    c /= np.linalg.norm(c)
    return c, orbs, I.pack_state(c, orbs)


@pytest.fixture(scope="module", params=list(SYSTEMS))
def pair(request):
    from codyfortran_gb300.engine import Engine
    sp = SYSTEMS[request.param]()
    o = Oracle(sp)
    e = Engine(sp)
    c, orbs, st = _state(sp, o, 11)
    yield sp, o, e, c, orbs, st
    e.close()


def test_sizes_and_grid(pair):
    sp, o, e, c, orbs, st = pair
    assert (e.nG, e.nO, e.nOS, e.nC) == (o.nG, o.nO, o.nOS, o.nC)
    assert rel(e.x, o.x) < 1e-15 and rel(e.w, o.w) < 1e-15


def test_configlist_tables_bit_exact(pair):
    sp, o, e, c, orbs, st = pair
    for bt in range(sp.n_bt):
        for kind in (0, 1):
            a, b = e.tables(bt, kind), o.tables(bt, kind)
            assert np.array_equal(a["codes"], b["codes"])
            assert np.array_equal(a["n_connected"], b["n_connected"])
            for key in ("excited_c", "orb_code", "factor"):
                assert a[key].shape == b[key].shape, key
                assert np.array_equal(a[key], b[key]), key


def test_single_body_op_and_h1(pair):
    sp, o, e, c, orbs, st = pair
    for t in (0.0, 3.7):
        d_gpu, h1_gpu = e.apply_single_body_op(orbs, t, want_h1=True)
        d_orc, h1_orc = o.apply_single_body_op(orbs, t, want_h1=True)
        assert rel(d_gpu, d_orc) < TOL
        assert rel(h1_gpu, h1_orc) < TOL
        assert rel(e.fill_h1(orbs, t), o.fill_h1(orbs, t)) < TOL


def test_sys_operators_on_one_orbital(pair):
    """The Sys* procedure pointers (kinetic, external potential with the laser,
    interaction source / potential / multiply) against the oracle."""
    sp, o, e, c, orbs, st = pair
    n_bt = sp.n_bt
    a, b = orbs[:, 0], orbs[:, -1]
    for bt in range(1, n_bt + 1):
        assert rel(e.sys_kinetic_multiply(b, 1.3, bt), o.kinetic_apply(b, 0 if sp.restricted else bt - 1)) < TOL
    for t in (0.0, 3.7):
        V = e.sys_potential_fill(t)
        Vo = o.potential() + o.field(t) * o.x
        assert rel(V, Vo) < TOL and np.all(V.imag == 0.0)
        assert rel(e.sys_potential_multiply(V, a), Vo * a) < TOL
    src = e.sys_interaction_src(a, b)
    assert rel(src, np.conj(a) * b * o.w) < TOL
    W = e.sys_interaction_potential(src)
    assert rel(W, o.interaction_potential(a, b)) < TOL
    assert rel(e.sys_interaction_multiply(W, b), W * b) < TOL


def test_rdms(pair):
    sp, o, e, c, orbs, st = pair
    assert rel(e.rdm1(c), o.rdm1(c)) < TOL
    assert rel(e.rdm2(c), o.rdm2(c)) < TOL


def test_ci_apply(pair):
    sp, o, e, c, orbs, st = pair
    rng = np.random.default_rng(5)
    n = o.nO
    h1 = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    h2 = rng.normal(size=(n, n, n, n)) + 1j * rng.normal(size=(n, n, n, n))
    assert rel(e.apply_h1(c, h1), o.apply_h1(c, h1)) < TOL
    assert rel(e.apply_h2(c, h2), o.apply_h2(c, h2)) < TOL


def test_fill_h2(pair):
    sp, o, e, c, orbs, st = pair
    assert rel(e.fill_h2(orbs, 0.0), o.fill_h2(orbs, 0.0)) < TOL


def test_correlation_op(pair):
    sp, o, e, c, orbs, st = pair
    r1, r2 = o.rdm1(c), o.rdm2(c)
    d_gpu, h2_gpu = e.apply_correlation_op(orbs, r1, r2, 0.0)
    d_orc, h2_orc = o.apply_correlation_op(orbs, r1, r2, 0.0)
    assert rel(d_gpu, d_orc) < TOL
    assert rel(h2_gpu, h2_orc) < TOL


def test_projectors(pair):
    sp, o, e, c, orbs, st = pair
    rng = np.random.default_rng(9)
    d = rng.normal(size=orbs.shape) + 1j * rng.normal(size=orbs.shape)
    assert rel(e.project_orbs(d, orbs), o.project_orbs(d, orbs)) < TOL
    raw = np.asfortranarray(rng.normal(size=orbs.shape) + 1j * rng.normal(size=orbs.shape))
    assert rel(e.orthonormalize(raw), o.orthonormalize(raw)) < TOL


@pytest.mark.parametrize("which", ["full", "orbs_lin", "nonlin"])
def test_time_derivative(pair, which):
    sp, o, e, c, orbs, st = pair
    t = 2.5
    assert rel(e.time_derivative(st, t, which), o.time_derivative(st, t, which)) < TOL


def test_energy(pair):
    sp, o, e, c, orbs, st = pair
    ea, eb = e.energy(st, 1.0), o.energy(st, 1.0)
    assert abs(ea - eb) <= TOL * abs(eb)


def test_rk4_nonlin(pair):
    sp, o, e, c, orbs, st = pair
    assert rel(e.rk(st, 0.3, 0.32), o.rk(st, 0.3, 0.32)) < TOL


def test_sil_fixed_order_with_metric(pair):
    sp, o, e, c, orbs, st = pair
    m = o.metric_weights()
    a = e.sil(st, 1.0, 1.01, 8, 0.0, 0, metric=m)
    b = o.sil(st, 1.0, 1.01, 8, 0.0, 0, metric=m)
    assert rel(a, b) < TOL


def test_sil_adaptive_euclidean(pair):
    sp, o, e, c, orbs, st = pair
    a = e.sil(st, 0.0, 0.05, 12, 1e-10, 8)
    b = o.sil(st, 0.0, 0.05, 12, 1e-10, 8)
    assert rel(a, b) < TOL


def test_split2_steps(pair):
    sp, o, e, c, orbs, st = pair
    a, b = st.copy(), st.copy()
    m = o.metric_weights()
    t, dt = 0.0, 0.01
    for _ in range(3):
        a = e.propagate_split2(a, t, t + dt, krylov_dim=10, use_metric=True)
        b = o.propagate_split2(b, t, t + dt, krylov_dim=10, metric=m)
        t += dt
    assert rel(a, b) < TOL


def test_resident_propagation_matches_host_api(pair):
    sp, o, e, c, orbs, st = pair
    a = st.copy()
    t, dt = 0.0, 0.01
    for _ in range(2):
        a = e.propagate_split2(a, t, t + dt, krylov_dim=10, use_metric=True)
        t += dt
    e.upload(st)
    e.propagate_resident(0.0, dt, 2, 10, use_metric=True)
    assert rel(e.download(), a) < 1e-14
    # one captured step replayed as a CUDA graph
    e.upload(st)
    e.propagate_resident(0.0, dt, 2, 10, use_metric=True, use_graph=True)
    assert rel(e.download(), a) < 1e-13


# ---------------------------------------------------------------------------
# Full-size and golden checks
# ---------------------------------------------------------------------------
def test_trimer_large_nonlin_full_size():
    """One NonLin derivative at the large workload (2801 points, 8008 determinants)."""
    from codyfortran_gb300.engine import Engine
    sp = S.cfg_trimer_large()
    o = Oracle(sp)
    e = Engine(sp)
    c, orbs, st = _state(sp, o, 7)
    a = e.time_derivative(st, 5.0, "nonlin")
    b = o.time_derivative(st, 5.0, "nonlin")
    assert rel(a, b) < TOL
    assert rel(e.tables(0, 1)["orb_code"], o.tables(0, 1)["orb_code"]) == 0.0
    e.close()


def test_he1d_golden_chain_on_gpu(golden):
    """He1d_04 relaxation (Euler + normalise + MGS x2) and He1d_06 SIL+RK4 real time on the GPU."""
    from codyfortran_gb300.engine import Engine
    sp = S.he1d_findiff((4, 4), False)
    e = Engine(sp)
    orbs = I.orthonormalize_state_orbitals(sp, I.harmonic_orbitals(sp, e.x), e.w)
    st = I.pack_state(I.unary_coeffs(sp), orbs)
    nC = e.nC
    en, conv, time = 0.0, 1e10, 0.0
    for _ in range(1000):
        if abs(conv) <= 1e-12:
            break
        for _ in range(10):
            st = e.rk(st, time, time + 0.01, integrator="euler", which="full", imag=True)
            time += 0.01
            st[:nC] = e.normalize_coeffs(st[:nC])
            o = e.orthonormalize(st[nC:].reshape(-1, e.nG).T)
            st[nC:] = o.ravel(order="F")
        old, en = en, e.energy(st, time)
        conv = en - old
    g04 = golden["he1d_04_mctdhf_imag"]["checks"][0]["golden"]
    assert abs(en - g04) < 1e-8
    e0, n0 = e.energy(st, 0.0), np.linalg.norm(st)
    t, dt = 0.0, 0.00002 / 2
    while t < 0.001:
        for _ in range(2):
            st = e.propagate_split2(st, t, t + dt, krylov_dim=24, tol=1e-12, max_restarts=8)
            t = t + dt
    en = e.energy(st, t)
    g05 = golden["he1d_05_mctdhf_split_rk4"]["checks"][0]["golden"]
    assert abs((en - e0) - (g05 - g04)) < 1e-10
    assert abs(en - g05) < 1e-7
    assert abs(np.linalg.norm(st) - n0) < 1e-10
    e.close()


def test_tdci_exact_diag_on_gpu(golden):
    """He1d_02: TDCI with all 21+21 grid-point orbitals gives the exact ground state."""
    from codyfortran_gb300.engine import Engine
    sp = S.he1d_findiff(n_orbs=(21, 21))
    sp.method = "tdci"
    e = Engine(sp)
    e.tdci_set_orbitals(I.grid_point_orbitals(sp, e.w))
    n = e.nC
    H = np.zeros((n, n), dtype=complex)
    for j in range(n):
        v = np.zeros(n, dtype=complex)
        v[j] = 1.0
        H[:, j] = 1j * e.time_derivative(v, 0.0, "tdci")
    e0 = np.linalg.eigvalsh(H)[0]
    assert abs(e0 - golden["he1d_02_tdci_exact_diag"]["checks"][0]["golden"]) < 1e-12
    e.close()
