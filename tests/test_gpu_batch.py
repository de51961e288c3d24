"""Batched trajectories (cgpu_batch_*): uneven systems advanced together (every
kernel covers all systems, one graph launch per step) must give what each
system gives alone, and the FP64 batch must match the CPU oracle."""
import numpy as np
import pytest

from oracle import Oracle
from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(np.ravel(b))
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / (nb if nb > 0 else 1.0)


def _small_helium():
    sp = S.helium_fedvr(20, 6, 4, laser=S.sin2_pulse(0.0534, omega=0.2, n_cycles=2.0, cep=0.3))
    sp.xmin, sp.xmax = -20.0, 20.0
    return sp


def _two_per_spin():
    sp = S.helium_fedvr(12, 6, 5, laser=S.sin2_pulse(0.03, omega=0.25, n_cycles=2.0, cep=1.0))
    sp.xmin, sp.xmax = -12.0, 12.0
    sp.n_bodies = (2, 2)
    return sp


def _states(engines, seed):
    out = []
    for k, e in enumerate(engines):
        rng = np.random.default_rng(seed + k)
        orbs = I.seeded_gaussian_orbitals(e.spec, e.x, e.w, seed + k)
        c = rng.normal(size=e.nC) + 1j * rng.normal(size=e.nC)
        c /= np.linalg.norm(c)
        out.append(I.pack_state(c, orbs))
    return out


# FP64: the batch sums its reductions over other block counts than a single
# system, so agreement is to rounding.  Mixed: the split-K partitions of the
# FP32-accumulated contractions differ too, so agreement is to the mixed form's
# own accuracy.  mixed_fx: the batch's digit width follows its longest grid
# (6-bit digits) while a small system alone uses 7- or 8-bit ones, so agreement
# is to the fixed-point form's truncation (~3e-9 per NonLin evaluation; these
# random states after 6 steps differ by up to ~1.5e-8; 2^6 less for mixed_fx6).
@pytest.mark.parametrize("precision,tol,etol", [("fp64", 1e-12, 1e-12), ("mixed", 2e-5, 1e-6),
                                                 ("mixed_fx", 5e-8, 1e-9), ("mixed_fx6", 1e-9, 1e-10)])
def test_batch_matches_individual_contexts(precision, tol, etol):
    from codyfortran_gb300.engine import Batch, Engine
    specs = S.batch_trajectory_specs(512, 1234)[:3] + [_small_helium(), _two_per_spin()]
    b = Batch(specs, precision, max_krylov=16)
    st = _states(b.systems, 5)
    b.upload(st)
    t0 = np.array([0.0, 3.0, 7.5, 1.0, 0.25])
    dt, n, K = 0.02, 3, 12
    assert b.propagate(t0, dt, n, K) > 0.0
    assert b.kernels_per_step() > 0
    # a second call continues from the advanced states on the same batch graph
    b.propagate(t0 + n * dt, dt, n, K)
    got = b.download()
    E = b.energies(t0 + 2 * n * dt)
    for k, sp in enumerate(specs):
        e = Engine(sp, precision, max_krylov=16)
        e.upload(st[k])
        e.propagate_resident(t0[k], dt, 2 * n, K, use_metric=True, use_graph=True)
        ref = e.download()
        e_ref = e.energy_resident(t0[k] + 2 * n * dt)
        e.close()
        assert rel(got[k], ref) <= tol, (k, rel(got[k], ref))
        assert abs(E[k] - e_ref) <= etol * abs(e_ref), (k, E[k], e_ref)
    b.close()


def test_batch_fp64_matches_oracle():
    from codyfortran_gb300.engine import Batch
    specs = [_small_helium(), _two_per_spin()]
    b = Batch(specs, "fp64")
    st = _states(b.systems, 17)
    b.upload(st)
    t0 = np.array([0.5, 0.0])
    dt, n, K = 0.01, 3, 10
    b.propagate(t0, dt, n, K, use_metric=True)
    got = b.download()
    for k, sp in enumerate(specs):
        o = Oracle(sp)
        m = o.metric_weights()
        s, t = st[k].copy(), t0[k]
        for _ in range(n):
            s = o.propagate_split2(s, t, t + dt, krylov_dim=K, metric=m)
            t += dt
        assert rel(got[k], s) < 1e-11, (k, rel(got[k], s))
    b.close()


@pytest.mark.parametrize("window", [1, 2, 3])
def test_krylov_window_matches_full_reorthogonalisation(window):
    """SIL with the three-term recurrence (window 1) or Gram-Schmidt against the
    last `window` Krylov vectors only, against the reference's loop over the
    whole basis: the same propagation to rounding for K = 12."""
    from codyfortran_gb300.engine import Batch
    specs = S.batch_trajectory_specs(512, 1234)[:3] + [_small_helium(), _two_per_spin()]
    full = Batch(specs, "fp64", max_krylov=12)
    loc = Batch(specs, "fp64", max_krylov=12, krylov_window=window)
    st = _states(full.systems, 23)
    full.upload(st)
    loc.upload(st)
    t0 = np.array([0.0, 3.0, 7.5, 1.0, 0.25])
    full.propagate(t0, 0.02, 4, 12)
    loc.propagate(t0, 0.02, 4, 12)
    a, b = full.download(), loc.download()
    for k in range(len(specs)):
        assert rel(b[k], a[k]) < 1e-13, (k, rel(b[k], a[k]))
    full.close()
    loc.close()


def test_krylov_window_rejects_negative():
    from codyfortran_gb300.engine import Batch, CodyError
    with pytest.raises(CodyError):
        Batch([_small_helium()], "fp64", krylov_window=-1)


def test_mixed_fx_batch_without_shared_interaction():
    """Systems whose interaction matrices are not blocks of one matrix (another
    softening) keep one interaction matrix per trajectory."""
    from codyfortran_gb300.engine import Batch, Engine
    other = _small_helium()
    other.int_s1 = 0.7
    specs = [_small_helium(), other, _two_per_spin()]
    b = Batch(specs, "mixed_fx", max_krylov=12)
    st = _states(b.systems, 31)
    b.upload(st)
    t0 = np.array([0.0, 1.0, 2.0])
    b.propagate(t0, 0.02, 3, 12)
    got = b.download()
    for k, sp in enumerate(specs):
        e = Engine(sp, "mixed_fx", max_krylov=12)
        e.upload(st[k])
        e.propagate_resident(t0[k], 0.02, 3, 12, use_metric=True, use_graph=True)
        ref = e.download()
        e.close()
        assert rel(got[k], ref) <= 1e-10, (k, rel(got[k], ref))
    b.close()


def test_mixed_fx_shared_interaction_matches_per_trajectory():
    """These grids nest (FEDVR elements of width 2 on boxes of different length),
    so the batch reads one shared interaction matrix at each trajectory's row
    offset.  Adding a system with another softening switches the batch to one
    matrix per trajectory with the same digit widths: the fixed-point
    contractions are exact sums of the same digits, so both batches agree to
    the rounding of their FP64 parts."""
    from codyfortran_gb300.engine import Batch
    specs = S.batch_trajectory_specs(512, 1234)[:3] + [_small_helium(), _two_per_spin()]
    other = _small_helium()
    other.int_s1 = 0.7
    shared = Batch(specs, "mixed_fx", max_krylov=12, krylov_window=2)
    single = Batch(specs + [other], "mixed_fx", max_krylov=12, krylov_window=2)
    assert shared.shared_interactions() >= 1 and single.shared_interactions() == 0
    st = _states(shared.systems, 41)
    st_other = _states(single.systems[-1:], 99)
    shared.upload(st)
    single.upload(st + st_other)
    t0 = np.array([0.0, 3.0, 7.5, 1.0, 0.25])
    shared.propagate(t0, 0.02, 4, 12)
    single.propagate(np.append(t0, 0.5), 0.02, 4, 12)
    a, b = shared.download(), single.download()
    Ea = shared.energies(t0 + 0.08)
    Eb = single.energies(np.append(t0, 0.5) + 0.08)
    for k in range(len(specs)):
        assert rel(a[k], b[k]) < 1e-12, (k, rel(a[k], b[k]))
        assert abs(Ea[k] - Eb[k]) <= 1e-12 * abs(Eb[k]), (k, Ea[k], Eb[k])
    shared.close()
    single.close()


def test_pinned_host_buffers():
    """Page-locked buffers from cgpu_host_alloc: batch upload / download and an
    in-place propagate_split2 give bit for bit what ordinary arrays give.  Each
    arm runs on a fresh context: the rho^-1 eigensolver starts from the previous
    call's eigenvectors, so a second run on the same context may differ in the
    last bits."""
    from codyfortran_gb300.engine import Batch, Engine, pinned_empty
    specs = [_small_helium(), _two_per_spin()]
    outs = []
    for pinned in (True, False):
        b = Batch(specs, "fp64")
        packed = b.pack(_states(b.systems, 7))
        src = packed
        if pinned:
            src = pinned_empty(packed.size)
            src[:] = packed
        b.upload(src)
        b.propagate(np.zeros(2), 0.02, 2, 10)
        dst = pinned_empty(packed.size) if pinned else None
        outs.append(b.download_packed(dst).copy())
        b.close()
    assert np.array_equal(outs[0], outs[1])
    e = Engine(specs[0])
    st = _states([e], 9)[0]
    ref = e.propagate_split2(st, 0.0, 0.02, krylov_dim=10, use_metric=True)
    e.close()
    e = Engine(specs[0])
    buf = pinned_empty(e.nS)
    buf[:] = st
    e.propagate_split2(buf, 0.0, 0.02, krylov_dim=10, use_metric=True, out=buf)
    e.close()
    assert np.array_equal(buf, ref)
    assert pinned_empty(0).size == 0
