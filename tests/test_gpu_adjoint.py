"""Pulse gradient (cgpu_tdci_adjoint) for the 1D helium pulse-optimisation
system: 100 x 6 FEDVR points, M=8 restricted orbitals (64 configurations),
4000 field samples of dt = 0.05 drawn N(0, 0.01^2) from seed 99.

* the adjoint gradient equals central finite differences (h = 1e-5) of the
  same discrete propagation on 32 random samples to 1e-6 relative to the
  gradient's magnitude (the finite differences carry ~1e-10 absolute rounding
  noise: J to ~1e-15 over 2h = 2e-5);
* it equals a host restatement of the same adjoint sweep to 1e-10;
* the forward map equals a host restatement of the same RK4 steps built from
  the engine's own TDCI time derivative (1e-12);
* the gradient does not depend on the checkpoint interval."""
import numpy as np
import pytest

from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S

pytestmark = pytest.mark.gpu

DT = 0.05


@pytest.fixture(scope="module")
def system():
    from codyfortran_gb300.engine import Engine
    sp = S.cfg_adjoint_helium(seed=99, n_samples=4000, dt=DT)
    sp.method = "tdci"
    e = Engine(sp)
    orbs = I.mgs_orthonormalize(I.harmonic_orbitals(sp, e.x), e.w)
    e.tdci_set_orbitals(orbs)
    n = e.nC

    def dense(t):
        H = np.zeros((n, n), dtype=complex)
        for j in range(n):
            v = np.zeros(n, dtype=complex)
            v[j] = 1.0
            H[:, j] = 1j * e.time_derivative(v, t, "tdci")
        return H

    A = dense(-1.0)                       # before the samples start: zero field
    E = np.asarray(sp.laser.samples, dtype=np.float64)
    X = (dense(0.5 * DT) - A) / E[0]      # step 0 carries E_0
    c0 = np.linalg.eigh(A)[1][:, 0].astype(complex)
    yield e, A, X, E, c0
    e.close()


def _host_forward(A, X, E, c0, n_steps):
    C = c0.copy()
    for n in range(n_steps):
        # one RK4 step of dC/dt = -i H_n C: C + zC + z^2C/2 + z^3C/6 + z^4C/24, z = -i dt H_n
        z = -1j * DT * (A + E[n] * X)
        u, s, fac = C.copy(), C.copy(), 1.0
        for p in range(1, 5):
            u = z @ u
            fac *= p
            s = s + u / fac
        C = s
    a = np.vdot(c0, C)
    return 1.0 - abs(a) ** 2, a, C


def test_forward_matches_host_restatement(system):
    e, A, X, E, c0 = system
    n = 200
    J, a, CN, _ = e.tdci_adjoint(c0, E[:n], DT, gradient=False)
    Jh, ah, Ch = _host_forward(A, X, E, c0, n)
    assert np.linalg.norm(CN - Ch) / np.linalg.norm(Ch) < 1e-12
    assert abs(a - ah) < 1e-12
    assert abs(J - Jh) < 1e-12


def test_adjoint_gradient_matches_finite_differences(system):
    e, A, X, E, c0 = system
    J, a, CN, g = e.tdci_adjoint(c0, E, DT, checkpoint=64)
    assert np.all(np.isfinite(g)) and 0.0 <= J < 1.0
    rng = np.random.default_rng(7)
    idx = rng.choice(len(E), size=32, replace=False)
    h = 1e-5
    scale = np.max(np.abs(g))
    assert scale > 0.0
    for n in idx:
        Ep, Em = E.copy(), E.copy()
        Ep[n] += h
        Em[n] -= h
        Jp = e.tdci_adjoint(c0, Ep, DT, gradient=False)[0]
        Jm = e.tdci_adjoint(c0, Em, DT, gradient=False)[0]
        fd = (Jp - Jm) / (2 * h)
        assert abs(g[n] - fd) <= 1e-6 * scale, (int(n), g[n], fd)


def _host_adjoint(A, X, E, c0, n_steps):
    """The adjoint sweep restated with dense numpy algebra (no checkpoints)."""
    C, Cs = c0.copy(), []
    for n in range(n_steps):
        Cs.append(C)
        z = -1j * DT * (A + E[n] * X)
        u, s, fac = C.copy(), C.copy(), 1.0
        for p in range(1, 5):
            u = z @ u
            fac *= p
            s = s + u / fac
        C = s
    a = np.vdot(c0, C)
    mu, g, fact = c0.copy(), np.zeros(n_steps), [1, 1, 2, 6, 24]
    for n in range(n_steps - 1, -1, -1):
        z = -1j * DT * (A + E[n] * X)
        u = [Cs[n]]
        for _ in range(3):
            u.append(z @ u[-1])
        w = [mu]
        for _ in range(4):
            w.append(z.conj().T @ w[-1])
        da = -1j * DT * sum(np.vdot(w[m], X @ u[q]) / fact[m + q + 1] for m in range(4) for q in range(4 - m))
        g[n] = -2.0 * np.real(np.conj(a) * da)
        mu = sum(w[m] / fact[m] for m in range(5))
    return 1.0 - abs(a) ** 2, g


def test_adjoint_matches_host_adjoint(system):
    e, A, X, E, c0 = system
    n = 1000
    J, a, CN, g = e.tdci_adjoint(c0, E[:n], DT, checkpoint=64)
    Jh, gh = _host_adjoint(A, X, E, c0, n)
    assert abs(J - Jh) < 1e-12
    assert np.max(np.abs(g - gh)) <= 1e-10 * np.max(np.abs(gh))


def test_adjoint_checkpoint_interval_irrelevant(system):
    e, A, X, E, c0 = system
    g64 = e.tdci_adjoint(c0, E[:700], DT, checkpoint=64)[3]
    g7 = e.tdci_adjoint(c0, E[:700], DT, checkpoint=7)[3]
    assert np.max(np.abs(g64 - g7)) <= 1e-13 * np.max(np.abs(g64))
