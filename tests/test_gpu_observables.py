"""On-device observables (cgpu_observables / cgpu_batch_observables), the GPU
imaginary-time relaxation (cgpu_relax) against the CPU oracle, and restart
files in the reference's raw format (cgpu_save_restart / cgpu_load_restart)."""
import numpy as np
import pytest

from oracle import Oracle
from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S

pytestmark = pytest.mark.gpu


def _helium():
    sp = S.helium_fedvr(20, 6, 4, laser=S.sin2_pulse(0.0534, omega=0.2, n_cycles=2.0, cep=0.3))
    sp.xmin, sp.xmax = -20.0, 20.0
    return sp


def _state(sp, x, w, seed, nC):
    rng = np.random.default_rng(seed)
    orbs = I.seeded_gaussian_orbitals(sp, x, w, seed)
    c = rng.normal(size=nC) + 1j * rng.normal(size=nC)
    return I.pack_state(c / np.linalg.norm(c), orbs), orbs, c / np.linalg.norm(c)


def test_observables_match_oracle():
    from codyfortran_gb300.engine import Engine
    sp = _helium()
    o, e = Oracle(sp), Engine(sp)
    st, orbs, c = _state(sp, o.x, o.w, 3, o.nC)
    t = 7.3
    e.upload(st)
    obs = e.observables(t)
    assert abs(obs["energy"] - o.energy(st, t)) <= 1e-12 * abs(o.energy(st, t))
    assert abs(obs["norm"] - np.linalg.norm(c)) < 1e-13
    r1 = o.rdm1(c)
    n = e.nOS
    xs = (orbs.conj() * (o.x * o.w)[:, None]).T @ orbs          # spatial <phi_i| x |phi_j>_w
    X = np.zeros((2 * n, 2 * n), dtype=complex)
    X[:n, :n] = xs
    X[n:, n:] = xs
    dip = np.real(np.sum(X * r1.T))
    assert abs(obs["dipole"] - dip) <= 1e-12 * max(1.0, abs(dip))
    occ = np.sort(np.linalg.eigvalsh(r1[:n, :n] + r1[n:, n:]))[::-1]
    assert np.max(np.abs(obs["occupations"] - occ)) < 1e-12
    assert abs(np.sum(occ) - 2.0) < 1e-12                       # two electrons
    e.close()


def test_batch_observables_match_single_systems():
    from codyfortran_gb300.engine import Batch, Engine
    specs = S.batch_trajectory_specs(512, 1234)[:3] + [_helium()]
    b = Batch(specs, "fp64")
    states = [_state(sp, s.x, s.w, 11 + k, s.nC)[0] for k, (sp, s) in enumerate(zip(specs, b.systems))]
    b.upload(states)
    t = np.array([0.0, 12.5, 3.0, 7.3])
    E, N, D, O = b.observables(t)
    for k, sp in enumerate(specs):
        e = Engine(sp)
        e.upload(states[k])
        ob = e.observables(t[k])
        e.close()
        assert abs(E[k] - ob["energy"]) <= 1e-12 * abs(ob["energy"])
        assert abs(N[k] - ob["norm"]) < 1e-13
        assert abs(D[k] - ob["dipole"]) <= 1e-12 * max(1.0, abs(ob["dipole"]))
        n = len(ob["occupations"])
        assert np.max(np.abs(O[k, :n] - ob["occupations"])) < 1e-12
        assert np.all(O[k, n:] == 0.0)
    b.close()


def test_relax_matches_oracle_and_golden(golden):
    """He1d_04 (unrestricted MCTDHF, 21-point grid): relaxation entirely on the GPU."""
    from codyfortran_gb300.engine import Engine
    sp = S.he1d_findiff((4, 4), False)
    o, e = Oracle(sp), Engine(sp)
    orbs = I.orthonormalize_state_orbitals(sp, I.harmonic_orbitals(sp, e.x), e.w)
    st = I.pack_state(I.unary_coeffs(sp), orbs)
    eg, sg, ng = e.relax(st, 0.01, 10, 1e-12, 1000)
    eo, so, no = o.relax(st, 0.01, 10, 1e-12, 1000)
    assert ng == no
    assert abs(eg - eo) < 1e-11
    g04 = golden["he1d_04_mctdhf_imag"]["checks"][0]["golden"]
    assert abs(eg - g04) < 1e-8
    e.close()


def test_restart_files_round_trip(tmp_path):
    from codyfortran_gb300.engine import Engine
    sp = S.he1d_findiff((4, 4), False)             # unrestricted: two body types of orbital files
    e = Engine(sp)
    st, orbs, c = _state(sp, e.x, e.w, 5, e.nC)
    e.upload(st)
    e.save_restart(tmp_path, with_rdm2=True)
    coeffs = np.fromfile(tmp_path / "coeffs.in", dtype=np.complex128)
    assert np.array_equal(coeffs, st[:e.nC])
    i1 = 0
    for bt in range(2):
        for k in range(4):
            f = np.fromfile(tmp_path / f"orb{bt + 1:02d}_{k + 1:02d}.in", dtype=np.complex128)
            assert np.array_equal(f, st[e.nC + i1 * e.nG:e.nC + (i1 + 1) * e.nG])
            i1 += 1
    r2 = e.rdm2(st[:e.nC])                          # nO^4, Fortran order
    blk = np.fromfile(tmp_path / "rdm2Bt01_02.in", dtype=np.complex128).reshape((4, 4, 4, 4), order="F")
    assert np.array_equal(blk, r2[0:4, 4:8, 0:4, 4:8])
    e2 = Engine(sp)
    e2.load_restart(tmp_path)
    assert np.array_equal(e2.download(), st)
    e.close()
    e2.close()


def test_batch_restart_files_match_single_system(tmp_path):
    """cgpu_batch_save_restart writes, per trajectory, the files a single
    context writes for the same state (bit for bit, rdm2 blocks included), and
    cgpu_batch_load_restart reads them back into every trajectory."""
    from codyfortran_gb300.engine import Batch, Engine
    specs = [S.he1d_findiff((4, 4), False), S.he1d_findiff((3, 3), False)]
    b = Batch(specs, "fp64")
    states = [_state(sp, s.x, s.w, 11 + k, s.nC)[0] for k, (sp, s) in enumerate(zip(specs, b.systems))]
    b.upload(states)
    b.save_restart(tmp_path, with_rdm2=True)
    for k, sp in enumerate(specs):
        one = tmp_path / f"single{k}"
        one.mkdir()
        e = Engine(sp)
        e.upload(states[k])
        e.save_restart(one, with_rdm2=True)
        e.close()
        names = sorted(p.name for p in one.iterdir())
        assert names == sorted(p.name for p in (tmp_path / f"traj{k:05d}").iterdir())
        assert any(n.startswith("rdm2Bt") for n in names)
        for n in names:
            assert (one / n).read_bytes() == (tmp_path / f"traj{k:05d}" / n).read_bytes(), (k, n)
    b2 = Batch(specs, "fp64")
    b2.load_restart(tmp_path)
    got = b2.download()
    for k in range(len(specs)):
        assert np.array_equal(got[k], states[k])
    b.close()
    b2.close()


def test_absorber_mask_and_per_step_application():
    from codyfortran_gb300.engine import Engine
    sp = _helium()
    onset, order = 12.0, 0.25
    ea, eb = Engine(sp), Engine(sp)
    st, orbs, c = _state(sp, ea.x, ea.w, 9, ea.nC)
    # one application against the mask restated on the host
    ea.absorber(onset, order)
    ea.upload(st)
    ea.absorber_apply()
    xi = np.abs(ea.x)
    t = (xi - onset) / (ea.x[-1] - onset)
    mask = np.where(xi < onset, 1.0, np.cos(0.5 * np.pi * t) ** (1.0 / order))
    ref = st.copy()
    ref[ea.nC:] = (orbs * mask[:, None]).ravel(order="F")
    got = ea.download()
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-14
    # applied after every step of the step graph == step, apply, step, apply
    ea.absorber(onset, order, apply_each_step=True)
    ea.upload(st)
    ea.propagate_resident(0.0, 0.01, 2, 10, use_metric=True, use_graph=True)
    eb.absorber(onset, order, apply_each_step=False)
    eb.upload(st)
    for k in range(2):
        eb.propagate_resident(0.01 * k, 0.01, 1, 10, use_metric=True, use_graph=True)
        eb.absorber_apply()
    a, b = ea.download(), eb.download()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-13
    ea.close()
    eb.close()


def test_tdci_sil_matches_oracle():
    """TDCI propagation of the CI vector alone by SIL (fixed orbitals, laser on)."""
    from codyfortran_gb300.engine import Engine
    sp = _helium()
    sp.method = "tdci"
    o, e = Oracle(sp), Engine(sp)
    orbs = I.mgs_orthonormalize(I.harmonic_orbitals(sp, e.x), e.w)
    o.tdci_set_orbitals(orbs)
    e.tdci_set_orbitals(orbs)
    rng = np.random.default_rng(4)
    c = rng.normal(size=e.nC) + 1j * rng.normal(size=e.nC)
    c /= np.linalg.norm(c)
    a, b, t = c.copy(), c.copy(), 1.0
    for _ in range(3):
        a = e.sil(a, t, t + 0.05, 12, which="tdci")
        b = o.sil(b, t, t + 0.05, 12, which="tdci")
        t += 0.05
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-12
    e.close()
