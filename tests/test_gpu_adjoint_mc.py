"""MCTDHF pulse gradient on the GPU (cgpu_mc_adjoint_forward / cgpu_mc_adjoint_backward).

* The adjoint's forward map is the Strang step of the engine and of the
  oracle with the same sampled field (1e-12), and its objective is
  1 - |<Psi_0|Psi_N>|^2 with the MCTDHF overlap computed on the host.
* The gradient equals the host restatement of the adjoint
  (tests/adjoint_reference.py, FP64 numpy) on a small system.
* On the 1D helium model of the pulse-optimisation workload (501 FEDVR points,
  M = 8 restricted orbitals, field samples N(0, 0.01^2) from seed 99,
  dt = 0.05, checkpoints every 64 steps) the gradient agrees with central
  differences (h = 1e-5) of the forward map on random samples within 1e-6 of
  the gradient's largest entry: 256 steps in the default suite, 1024 in a slow
  test.  The start (and reference) state has every natural orbital occupied
  (seed-42 orbitals, a seeded random CI vector).  From the relaxed ground state
  the Strang step of the reference is exponentially sensitive -- its
  natural occupations reach 7e-12 and rho^-1 makes the splitting error
  large: the exact gradient grows to 5e6 after 256 steps and 1.6e19 after
  1024 -- so central differences at h = 1e-5 leave the linear range there;
  that case is checked at 32 steps, where it is still linear.
"""
import numpy as np
import pytest

from oracle import Oracle
from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S
from adjoint_reference import Adjoint, Dense
from mctdhf_util import mctdhf_overlap

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _small(field, dt, n_el=8, m=3):
    sp = S.helium_fedvr(n_el, 6, m, laser=S.Laser(kind="sampled", samples=field, sample_dt=dt, sample_t0=0.0))
    sp.xmin, sp.xmax = -float(n_el), float(n_el)
    return sp


def _state(sp, x, w, seed):
    rng = np.random.default_rng(seed)
    n = sp.n_coeffs
    c = rng.normal(size=n) + 1j * rng.normal(size=n)
    return I.pack_state(c / np.linalg.norm(c), I.seeded_gaussian_orbitals(sp, x, w, seed))


def test_forward_map_is_the_strang_step():
    from codyfortran_gb300.engine import Engine
    nT, dt, K = 7, 0.05, 8
    field = np.random.default_rng(1).normal(0.0, 0.02, size=nT)
    sp = _small(field, dt)
    o, e = Oracle(sp), Engine(sp, max_krylov=K)
    st = _state(sp, o.x, o.w, 2)
    J, ov, fin = e.mc_adjoint_forward(st, field, dt, krylov_dim=K, checkpoint=3)
    m = o.metric_weights()
    a, b = st.copy(), st.copy()
    for n in range(nT):
        a = o.propagate_split2(a, n * dt, (n + 1) * dt, krylov_dim=K, metric=m)
        b = e.propagate_split2(b, n * dt, (n + 1) * dt, krylov_dim=K, use_metric=True)
    assert rel(fin, a) < 1e-12
    assert rel(fin, b) < 1e-12
    O = mctdhf_overlap(sp, o.nG, o.w, st, fin)
    assert abs(ov - O) < 1e-12
    assert abs(J - (1.0 - abs(O) ** 2)) < 1e-12
    e.close()


def test_gradient_matches_host_adjoint():
    from codyfortran_gb300.engine import Engine
    nT, dt, K = 12, 0.05, 8
    field = np.random.default_rng(99).normal(0.0, 0.01, size=nT)
    sp = _small(field, dt)
    o, e = Oracle(sp), Engine(sp, max_krylov=K)
    st = _state(sp, o.x, o.w, 3)
    X = o.x
    ref = Adjoint(Dense(o, 1.0 / np.sqrt((X[:, None] - X[None, :]) ** 2 + 1.0)), field, dt, K)
    Jr, Or, sNr, gr = ref.run(st, checkpoint=5)
    J, ov, fin = e.mc_adjoint_forward(st, field, dt, krylov_dim=K, checkpoint=5)
    g = e.mc_adjoint_backward()
    print(f"host J {Jr:.15f} GPU J {J:.15f}; gradient rel diff {rel(g, gr):.2e}")
    assert abs(J - Jr) < 1e-12
    assert rel(fin, sNr) < 1e-12
    assert rel(g, gr) < 1e-9
    # the gradient does not depend on the checkpoint interval
    e.mc_adjoint_forward(st, field, dt, krylov_dim=K, checkpoint=1)
    assert rel(e.mc_adjoint_backward(), g) < 1e-12
    e.close()


def _helium_m8(field, dt):
    return S.helium_fedvr(100, 6, 8, laser=S.Laser(kind="sampled", samples=field, sample_dt=dt, sample_t0=0.0))


def _fd_check(n_steps, n_idx, start):
    from codyfortran_gb300.engine import Engine
    dt, K, chk = 0.05, 12, 64
    field = np.random.default_rng(99).normal(0.0, 0.01, size=4000)[:n_steps]
    sp = _helium_m8(field, dt)
    e = Engine(sp, max_krylov=K)
    sp0 = _helium_m8(field, dt)
    sp0.laser = S.Laser()
    if start == "relaxed":
        # the field-free ground state: imaginary-time relaxation from seed-42 orbitals
        r = Engine(sp0)
        st0 = I.pack_state(I.unary_coeffs(sp0), I.seeded_gaussian_orbitals(sp0, r.x, r.w, 42))
        _, st, _ = r.relax(st0, 0.005, 10, 1e-12, 2000)
        r.close()
    else:
        st = _state(sp0, e.x, e.w, 42)
    J, ov, fin = e.mc_adjoint_forward(st, field, dt, krylov_dim=K, checkpoint=chk)
    g = e.mc_adjoint_backward()
    gmax = np.max(np.abs(g))
    idx = np.sort(np.random.default_rng(7).choice(n_steps, size=n_idx, replace=False))
    h = 1e-5
    worst = 0.0
    for n in idx:
        f1, f2 = field.copy(), field.copy()
        f1[n] += h
        f2[n] -= h
        fd = (e.mc_adjoint_forward(st, f1, dt, K, chk)[0] - e.mc_adjoint_forward(st, f2, dt, K, chk)[0]) / (2 * h)
        worst = max(worst, abs(fd - g[n]) / gmax)
    print(f"helium M=8, {start} start, {n_steps} steps: J {J:.6e}, max |dJ/dE| {gmax:.3e}, "
          f"worst |FD - adjoint| / max {worst:.2e} over {n_idx} samples")
    assert worst < 1e-6
    e.close()
    return g


def test_gradient_matches_finite_differences_helium_m8():
    _fd_check(256, 8, "correlated")


def test_gradient_matches_finite_differences_helium_m8_relaxed_start():
    _fd_check(32, 4, "relaxed")


@pytest.mark.slow
def test_gradient_matches_finite_differences_helium_m8_1024_samples():
    _fd_check(1024, 4, "correlated")
