"""Mixed-precision forms: tcgen05 split contractions against the FP64 oracle.

Tolerances state the accuracy of each form: bf16x3 (hi + lo operands, three
products, FP32 accumulation), bf16x6 (hi + mid + lo, six products), and the
fixed-point forms mixed_fx / mixed_fx6 (bf16 digit slices holding 30 / 36
bits of each operand row's maximum, exact per-level accumulation: only the
operand truncation remains).  The relative errors measured here are what the forms
deliver; the propagation check compares energy and norm of a mixed
trajectory with the FP64 one.
"""
import numpy as np
import pytest

from oracle import Oracle
from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S

pytestmark = pytest.mark.gpu

TOL = {"mixed": 2e-4, "mixed6": 2e-6, "mixed_fx": 1e-7, "mixed_fx6": 1e-9}
PRECISIONS = ["mixed", "mixed6", "mixed_fx", "mixed_fx6"]


def rel(a, b):
    return np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel()) / np.linalg.norm(np.asarray(b).ravel())


def _systems():
    he = S.helium_fedvr(20, 6, 4, laser=S.sin2_pulse(0.0534, omega=0.2, n_cycles=2.0))
    he.xmin, he.xmax = -20.0, 20.0
    one = S.SystemSpec(grid_kind="fedvr", xmin=-16.0, xmax=16.0, n_elements=16, n_locals=8, n_bodies=(3,),
                       n_orbs=(6,), masses=(1.0,), stats="f", nuclei=[S.Nucleus(-2.0, 1.5), S.Nucleus(2.0, 1.5)],
                       int_kind="dense")
    return {"helium_restricted": he, "single_body_type": one}


def _state(sp, o, seed):
    rng = np.random.default_rng(seed)
    orbs = I.seeded_gaussian_orbitals(sp, o.x, o.w, seed)
    c = rng.normal(size=o.nC) + 1j * rng.normal(size=o.nC)
    c /= np.linalg.norm(c)
    return c, orbs, I.pack_state(c, orbs)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", ["helium_restricted", "single_body_type"])
def test_mixed_correlation_and_nonlin(name, precision):
    from codyfortran_gb300.engine import Engine
    sp = _systems()[name]
    o = Oracle(sp)
    e = Engine(sp, precision=precision)
    c, orbs, st = _state(sp, o, 5)
    r1, r2 = o.rdm1(c), o.rdm2(c)
    d_gpu, h2_gpu = e.apply_correlation_op(orbs, r1, r2, 0.0)
    d_orc, h2_orc = o.apply_correlation_op(orbs, r1, r2, 0.0)
    print(f"{name} {precision}: correlation {rel(d_gpu, d_orc):.3e}, h2 {rel(h2_gpu, h2_orc):.3e}")
    assert rel(d_gpu, d_orc) < TOL[precision]
    assert rel(h2_gpu, h2_orc) < TOL[precision]
    assert rel(e.time_derivative(st, 1.5, "nonlin"), o.time_derivative(st, 1.5, "nonlin")) < TOL[precision]
    e.close()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_mixed_nonlin_full_size(precision):
    """2801 points, 16 orbitals (136 pairs), 8008 determinants."""
    from codyfortran_gb300.engine import Engine
    sp = S.cfg_trimer_large()
    o = Oracle(sp)
    e = Engine(sp, precision=precision)
    c, orbs, st = _state(sp, o, 7)
    a = e.time_derivative(st, 5.0, "nonlin")
    b = o.time_derivative(st, 5.0, "nonlin")
    err = rel(a, b)
    print(f"{precision}: NonLin relative error {err:.3e}")
    assert err < TOL[precision]
    e.close()


def _span_defect(a, b, nC, nG, n, w):
    """1 - |det <phi_a|phi_b>_w| of the stored orbitals of two states."""
    fa = a[nC:nC + nG * n].reshape(n, nG)
    fb = b[nC:nC + nG * n].reshape(n, nG)
    return abs(1.0 - abs(np.linalg.det((fa.conj() * w) @ fb.T)))


@pytest.mark.parametrize("precision", PRECISIONS)
def test_mixed_trajectory_energy_norm(precision):
    """Energy, norm, dipole and orbital span of a mixed-precision trajectory
    against the FP64 GPU trajectory."""
    from codyfortran_gb300.engine import Engine
    sp = S.cfg_helium_small()
    f = Engine(sp, precision="fp64")
    m = Engine(sp, precision=precision)
    orbs = I.seeded_gaussian_orbitals(sp, f.x, f.w, 42)
    st = I.pack_state(I.unary_coeffs(sp), orbs)
    f.upload(st)
    m.upload(st)
    n_steps, dt = 200, 0.01
    f.propagate_resident(0.0, dt, n_steps, 12, use_metric=True)
    m.propagate_resident(0.0, dt, n_steps, 12, use_metric=True)
    t = n_steps * dt
    ef, em = f.energy_resident(t), m.energy_resident(t)
    sf, sm = f.download(), m.download()
    w = f.metric_weights()
    nf, nm = np.sqrt(np.sum(np.abs(sf) ** 2 * w)), np.sqrt(np.sum(np.abs(sm) ** 2 * w))
    de, dn = abs(em - ef) / abs(ef), abs(nm - nf)
    dx = abs(m.observables(t)["dipole"] - f.observables(t)["dipole"])
    print(f"{precision}: {n_steps} steps, |dE|/|E| = {de:.3e}, |d norm| = {dn:.3e}, |d<x>| = {dx:.3e}")
    # measured on GB300 over these 200 steps: |dE|/|E| 1.2e-6 / 1.2e-7 / 2.5e-10 / 2.3e-12,
    # |d<x>| 1.3e-4 / 4.4e-6 / 7.2e-9 / 1.7e-10 (bf16x3, bf16x6, fx, fx6)
    lim = {"mixed": (1e-5, 1e-6, 1e-3), "mixed6": (2e-6, 2e-7, 5e-5), "mixed_fx": (1e-8, 1e-9, 1e-7),
           "mixed_fx6": (1e-9, 1e-10, 2e-9)}[precision]
    assert de < lim[0] and dn < lim[1] and dx < lim[2]
    f.close()
    m.close()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_mixed_trajectory_orbital_span(precision):
    """1 - |det <phi_mixed|phi_FP64>_w| from a random CI vector (every orbital
    occupied).  From a single determinant the empty orbitals are fixed only
    through the regularised rho^-1, and their span differs between any two
    runs (2.7e-3 for every form here, FP64-level forms included), so the
    span is compared where all orbitals carry weight."""
    from codyfortran_gb300.engine import Engine
    sp = S.cfg_helium_small()
    f = Engine(sp, precision="fp64")
    m = Engine(sp, precision=precision)
    rng = np.random.default_rng(5)
    c = rng.normal(size=f.nC) + 1j * rng.normal(size=f.nC)
    st = I.pack_state(c / np.linalg.norm(c), I.seeded_gaussian_orbitals(sp, f.x, f.w, 42))
    f.upload(st)
    m.upload(st)
    n_steps, dt = 50, 0.01
    f.propagate_resident(0.0, dt, n_steps, 12, use_metric=True)
    m.propagate_resident(0.0, dt, n_steps, 12, use_metric=True)
    t = n_steps * dt
    ds = _span_defect(m.download(), f.download(), f.nC, f.nG, f.nOS, f.w)
    de = abs(m.energy_resident(t) - f.energy_resident(t)) / abs(f.energy_resident(t))
    print(f"{precision}: {n_steps} steps from a random CI vector, span defect = {ds:.3e}, |dE|/|E| = {de:.3e}")
    assert ds < 1e-9
    f.close()
    m.close()


@pytest.mark.slow
def test_mixed_fx6_batch_horizon_1500_steps():
    """The headline form over the whole batch horizon: the first 32 trajectories
    of the seed-1234 batch (uneven grids, orbital counts and pulses) advanced
    1500 steps of dt = 0.02 (K = 12) in mixed_fx6 and in FP64 from the same
    states; every 10 steps each trajectory's energy within 1e-8 relative and
    its norm within 1e-8 of the FP64 run."""
    import bench
    specs, cfg = bench.workload("batch512")
    rows = bench.accuracy_horizon(specs[:32], cfg, "mixed_fx6", 1500, every=10, window=1)
    e_max = max(r[1] for r in rows)
    n_max = max(r[4] for r in rows)
    a_max = max(r[7] for r in rows)
    f_max = max(r[8] for r in rows)
    worst = max(rows, key=lambda r: r[1])
    print(f"mixed_fx6 32 trajectories x 1500 steps: max |dE|/|E| {e_max:.3e} (step {worst[0]}, trajectory "
          f"{worst[5]}, |E| {worst[6]:.3e}), max |dE| {a_max:.3e} Eh, max |dE|/max(|E|, 1) {f_max:.3e}, "
          f"max |d||C||| {n_max:.3e}")
    assert f_max < 1e-8 and a_max < 1e-8 and n_max < 1e-8
