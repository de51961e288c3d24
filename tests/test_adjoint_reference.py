"""The host restatement of the MCTDHF pulse gradient (tests/adjoint_reference.py)
pinned on the CPU before it serves as the GPU adjoint's reference:

* its dense NonLin derivative equals the oracle's (configuration tables,
  generic RDMs, the reference's ApplyCorrelationOp) to 1e-13;
* its vector-Jacobian product agrees with central differences of the
  derivative in random state directions and in the field;
* its Strang step equals the oracle's with the same sampled field;
* its gradient of J = 1 - |<Psi_0|Psi_N>|^2 agrees with central differences.
"""
import numpy as np

from oracle import Oracle
from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S
from adjoint_reference import Adjoint, Dense


def _system(field=None, dt=0.05, n_el=6, m=3):
    laser = S.Laser(kind="sampled", samples=field, sample_dt=dt, sample_t0=0.0) if field is not None else \
        S.sin2_pulse(0.05, omega=0.3, n_cycles=2.0)
    sp = S.helium_fedvr(n_el, 6, m, laser=laser)
    sp.xmin, sp.xmax = -float(n_el), float(n_el)
    o = Oracle(sp)
    X = o.x
    D = Dense(o, 1.0 / np.sqrt((X[:, None] - X[None, :]) ** 2 + 1.0))
    rng = np.random.default_rng(3)
    c = rng.normal(size=m * m) + 1j * rng.normal(size=m * m)
    st = I.pack_state(c / np.linalg.norm(c), I.seeded_gaussian_orbitals(sp, o.x, o.w, 5))
    return sp, o, D, st


def test_dense_nonlin_matches_oracle():
    sp, o, D, st = _system(n_el=8, m=4)
    t = 2.3
    a, _ = D.forward(st, o.field(t))
    b = o.time_derivative(st, t, "nonlin")
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-13


def test_dense_vjp_matches_finite_differences():
    sp, o, D, st = _system()
    E = 0.037
    out, tape = D.forward(st, E)
    rng = np.random.default_rng(4)
    obar = rng.normal(size=out.size) + 1j * rng.normal(size=out.size)
    sbar, Ebar = D.vjp(tape, obar)
    h = 1e-6
    for _ in range(3):
        d = rng.normal(size=st.size) + 1j * rng.normal(size=st.size)
        fd = np.real(np.vdot(obar, (D.forward(st + h * d, E)[0] - D.forward(st - h * d, E)[0]) / (2 * h)))
        assert abs(fd - np.real(np.vdot(sbar, d))) < 1e-7 * abs(fd)
    fd = np.real(np.vdot(obar, (D.forward(st, E + h)[0] - D.forward(st, E - h)[0]) / (2 * h)))
    assert abs(fd - Ebar) < 1e-7 * abs(fd)


def test_strang_step_matches_oracle_and_gradient_matches_fd():
    nT, dt, K = 10, 0.05, 8
    field = np.random.default_rng(99).normal(0.0, 0.01, size=nT)
    sp, o, D, st = _system(field, dt)
    A = Adjoint(D, field, dt, K)
    a = st.copy()
    b = st.copy()
    m = o.metric_weights()
    for n in range(3):
        a, _ = A.step(a, n)
        b = o.propagate_split2(b, n * dt, (n + 1) * dt, krylov_dim=K, metric=m)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-13
    J, O, sN, grad = A.run(st, checkpoint=4)
    h = 1e-4
    for n in (0, 4, 9):
        f1, f2 = field.copy(), field.copy()
        f1[n] += h
        f2[n] -= h
        fd = (Adjoint(D, f1, dt, K).run(st, 4)[0] - Adjoint(D, f2, dt, K).run(st, 4)[0]) / (2 * h)
        assert abs(fd - grad[n]) < 1e-7 * abs(fd), (n, fd, grad[n])
