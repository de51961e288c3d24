"""ctypes wrapper of the CPU oracle (oracle/cody_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker that the GB300 engine's results are
compared against.  Imported by tests/, by __graft_entry__.smoke() and by the
cpu_baseline leg of bench.py; never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from codyfortran_gb300.spec import SystemSpec

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcodyoracle.so")


class OrcSpec(C.Structure):
    _fields_ = [
        ("grid_kind", C.c_int), ("xmin", C.c_double), ("xmax", C.c_double),
        ("n_points", C.c_int), ("n_elements", C.c_int), ("n_locals", C.c_int),
        ("xmin_excluded", C.c_int), ("xmax_excluded", C.c_int),
        ("n_bt", C.c_int), ("n_bodies", C.c_int * 4), ("n_orbs", C.c_int * 4), ("mass", C.c_double * 4),
        ("stats", C.c_char * 4), ("restricted", C.c_int), ("reg_eps", C.c_double),
        ("n_nuclei", C.c_int), ("nuc_pos", C.c_double * 8), ("nuc_charge", C.c_double * 8),
        ("nuc_s1", C.c_double * 8), ("nuc_s2", C.c_double * 8), ("nuc_damp", C.c_double * 8),
        ("has_interaction", C.c_int), ("int_strength", C.c_double), ("int_s1", C.c_double),
        ("int_s2", C.c_double), ("int_damp", C.c_double), ("int_kind", C.c_int),
        ("laser_kind", C.c_int), ("E0", C.c_double), ("omega", C.c_double), ("n_cycles", C.c_double),
        ("cep", C.c_double), ("t_start", C.c_double),
        ("field_samples", C.POINTER(C.c_double)), ("n_samples", C.c_int),
        ("sample_dt", C.c_double), ("sample_t0", C.c_double),
        ("method", C.c_int), ("n_threads", C.c_int),
    ]


def build() -> str:
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "cody_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_create.restype = C.c_void_p
        _lib.orc_create.argtypes = [C.POINTER(OrcSpec)]
        _lib.orc_field.restype = C.c_double
        _lib.orc_energy.restype = C.c_double
        _lib.orc_relax.restype = C.c_double
        for name in ["orc_destroy", "orc_sizes", "orc_grid", "orc_configlist_sizes", "orc_configlist_tables",
                     "orc_kinetic_apply", "orc_fedvr_second_derivative", "orc_fedvr_first_derivative", "orc_field",
                     "orc_potential", "orc_apply_single_body_op", "orc_fill_h1", "orc_fill_h2",
                     "orc_interaction_potential", "orc_apply_correlation_op", "orc_apply_h1_fill_rdm1",
                     "orc_apply_h2_fill_rdm2", "orc_project_coeffs", "orc_project_orbs", "orc_orthonormalize",
                     "orc_normalize", "orc_time_derivative", "orc_energy", "orc_tdci_set_orbitals",
                     "orc_integrate_rk", "orc_integrate_sil", "orc_propagate_split2", "orc_relax", "orc_error"]:
            getattr(_lib, name).argtypes = None
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)


def _d(v):
    return C.c_double(float(v))


_KIND = {"const": 0, "fedvr": 1}
_INTK = {"toeplitz": 0, "dense": 1}
_LASK = {"none": 0, "sin2": 1, "sampled": 2}


class Oracle:
    """CPU restatement of the reference hot path for one system."""

    def __init__(self, spec: SystemSpec, n_threads: int = 0):
        self.spec = spec
        s = OrcSpec()
        s.grid_kind = _KIND[spec.grid_kind]
        s.xmin, s.xmax = spec.xmin, spec.xmax
        s.n_points, s.n_elements, s.n_locals = spec.n_points, spec.n_elements, spec.n_locals
        s.xmin_excluded, s.xmax_excluded = int(spec.xmin_excluded), int(spec.xmax_excluded)
        s.n_bt = spec.n_bt
        for b in range(spec.n_bt):
            s.n_bodies[b] = int(spec.n_bodies[b])
            s.n_orbs[b] = int(spec.n_orbs[b])
            s.mass[b] = float(spec.masses[b])
        s.stats = spec.stats.encode()[:4]
        s.restricted = int(spec.restricted)
        s.reg_eps = spec.reg_eps
        s.n_nuclei = len(spec.nuclei)
        for i, n in enumerate(spec.nuclei):
            s.nuc_pos[i], s.nuc_charge[i] = n.position, n.charge
            s.nuc_s1[i], s.nuc_s2[i], s.nuc_damp[i] = n.softening1, n.softening2, n.dampening
        s.has_interaction = int(spec.has_interaction)
        s.int_strength, s.int_s1, s.int_s2, s.int_damp = spec.int_strength, spec.int_s1, spec.int_s2, spec.int_damp
        s.int_kind = _INTK[spec.int_kind]
        L = spec.laser
        s.laser_kind = _LASK[L.kind]
        s.E0, s.omega, s.n_cycles, s.cep, s.t_start = L.E0, L.omega, L.n_cycles, L.cep, L.t_start
        self._samples = None
        if L.kind == "sampled":
            self._samples = np.ascontiguousarray(L.samples, dtype=np.float64)
            s.field_samples = self._samples.ctypes.data_as(C.POINTER(C.c_double))
            s.n_samples = len(self._samples)
            s.sample_dt, s.sample_t0 = L.sample_dt, L.sample_t0
        s.method = 1 if spec.method == "tdci" else 0
        s.n_threads = n_threads
        self._s = s
        self.h = C.c_void_p(lib().orc_create(C.byref(s)))
        sz = (C.c_int * 5)()
        lib().orc_sizes(self.h, sz)
        self.nG, self.nO, self.nOS, self.nC, self.nBt = list(sz)
        self.x = np.zeros(self.nG)
        self.w = np.zeros(self.nG)
        lib().orc_grid(self.h, _p(self.x), _p(self.w))

    def __del__(self):
        try:
            lib().orc_destroy(self.h)
        except Exception:
            pass

    # sizes ---------------------------------------------------------------
    @property
    def n_state(self):
        return self.nC if self.spec.method == "tdci" else self.nC + self.nG * self.nOS

    def split(self, state):
        return state[: self.nC], state[self.nC:].reshape(self.nOS, self.nG).T

    # config tables -----------------------------------------------------
    def tables(self, bt, kind):
        sz = (C.c_int * 3)()
        lib().orc_configlist_sizes(self.h, C.c_int(bt), sz)
        n_conf, ms, md = list(sz)
        mc = ms if kind == 0 else md
        codes = np.zeros(n_conf, dtype=np.int64)
        ncon = np.zeros(n_conf, dtype=np.int32)
        exc = np.zeros(mc * n_conf, dtype=np.int32)
        oc = np.zeros(mc * n_conf, dtype=np.int32)
        fac = np.zeros(mc * n_conf, dtype=np.float64)
        lib().orc_configlist_tables(self.h, C.c_int(bt), C.c_int(kind), _p(codes), _p(ncon), _p(exc), _p(oc), _p(fac))
        f = lambda a: a.reshape(n_conf, mc).T  # (maxConn, nConf) column-major
        return dict(codes=codes, n_connected=ncon, excited_c=f(exc), orb_code=f(oc), factor=f(fac))

    # operators ---------------------------------------------------------
    def potential(self):
        v = np.zeros(self.nG)
        lib().orc_potential(self.h, _p(v))
        return v

    def field(self, t):
        return lib().orc_field(self.h, _d(t))

    def kinetic_apply(self, orb, bt=0):
        orb = np.ascontiguousarray(orb, dtype=np.complex128)
        out = np.zeros(self.nG, dtype=np.complex128)
        lib().orc_kinetic_apply(self.h, _p(orb), _p(out), C.c_int(bt))
        return out

    def fedvr_derivative(self, f, order=2):
        f = np.ascontiguousarray(f, dtype=np.complex128)
        out = np.zeros(self.nG, dtype=np.complex128)
        fn = lib().orc_fedvr_second_derivative if order == 2 else lib().orc_fedvr_first_derivative
        fn(self.h, _p(f), _p(out))
        return out

    def interaction_potential(self, orb_conj, orb):
        a = np.ascontiguousarray(orb_conj, dtype=np.complex128)
        b = np.ascontiguousarray(orb, dtype=np.complex128)
        out = np.zeros(self.nG, dtype=np.complex128)
        lib().orc_interaction_potential(self.h, _p(a), _p(b), _p(out))
        return out

    def _orbs(self, orbs):
        """(nG, nOS) -> Fortran-ordered contiguous buffer."""
        return np.asfortranarray(orbs, dtype=np.complex128)

    def apply_single_body_op(self, orbs, t, want_h1=False):
        o = self._orbs(orbs)
        d = np.zeros((self.nG, self.nOS), dtype=np.complex128, order="F")
        h1 = np.zeros((self.nO, self.nO), dtype=np.complex128, order="F") if want_h1 else None
        lib().orc_apply_single_body_op(self.h, _p(d), _p(o), _d(t), _p(h1))
        return (d, h1) if want_h1 else d

    def fill_h1(self, orbs, t):
        o = self._orbs(orbs)
        h1 = np.zeros((self.nO, self.nO), dtype=np.complex128, order="F")
        lib().orc_fill_h1(self.h, _p(h1), _p(o), _d(t))
        return h1

    def fill_h2(self, orbs, t):
        o = self._orbs(orbs)
        n = self.nO
        h2 = np.zeros((n, n, n, n), dtype=np.complex128, order="F")
        lib().orc_fill_h2(self.h, _p(h2), _p(o), _d(t))
        return h2

    def apply_correlation_op(self, orbs, rdm1, rdm2, t):
        o = self._orbs(orbs)
        r1 = np.asfortranarray(rdm1, dtype=np.complex128)
        r2 = np.asfortranarray(rdm2, dtype=np.complex128)
        d = np.zeros((self.nG, self.nOS), dtype=np.complex128, order="F")
        n = self.nO
        h2 = np.zeros((n, n, n, n), dtype=np.complex128, order="F")
        lib().orc_apply_correlation_op(self.h, _p(d), _p(o), _p(r1), _p(r2), _d(t), _p(h2))
        return d, h2

    def rdm1(self, coeffs):
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        r = np.zeros((self.nO, self.nO), dtype=np.complex128, order="F")
        lib().orc_apply_h1_fill_rdm1(self.h, _p(c), _p(r), None, None)
        return r

    def rdm2(self, coeffs):
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        n = self.nO
        r = np.zeros((n, n, n, n), dtype=np.complex128, order="F")
        lib().orc_apply_h2_fill_rdm2(self.h, _p(c), _p(r), None, None)
        return r

    def apply_h1(self, coeffs, h1):
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        h = np.asfortranarray(h1, dtype=np.complex128)
        d = np.zeros(self.nC, dtype=np.complex128)
        lib().orc_apply_h1_fill_rdm1(self.h, _p(c), None, _p(d), _p(h))
        return d

    def apply_h2(self, coeffs, h2):
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        h = np.asfortranarray(h2, dtype=np.complex128)
        d = np.zeros(self.nC, dtype=np.complex128)
        lib().orc_apply_h2_fill_rdm2(self.h, _p(c), None, _p(d), _p(h))
        return d

    def project_orbs(self, d_orbs, orbs):
        d = np.asfortranarray(d_orbs, dtype=np.complex128).copy(order="F")
        o = self._orbs(orbs)
        lib().orc_project_orbs(self.h, _p(d), _p(o))
        return d

    def orthonormalize(self, orbs):
        o = np.asfortranarray(orbs, dtype=np.complex128).copy(order="F")
        rc = lib().orc_orthonormalize(self.h, _p(o))
        if rc != 0:
            raise RuntimeError("Grid Orthonormalize: vector with non-positive norm")
        return o

    # state level -------------------------------------------------------
    def time_derivative(self, state, t, which="full"):
        w = {"full": 0, "orbs_lin": 1, "nonlin": 2, "tdci": 3}[which]
        s = np.ascontiguousarray(state, dtype=np.complex128)
        d = np.zeros_like(s)
        lib().orc_time_derivative(self.h, C.c_int(w), _p(d), _p(s), _d(t))
        return d

    def energy(self, state, t=0.0):
        s = np.ascontiguousarray(state, dtype=np.complex128)
        return lib().orc_energy(self.h, _p(s), _d(t))

    def tdci_set_orbitals(self, orbs):
        o = self._orbs(orbs)
        lib().orc_tdci_set_orbitals(self.h, _p(o))

    def rk(self, state, t0, t1, integrator="rk4", which="nonlin", imag=False):
        s = np.ascontiguousarray(state, dtype=np.complex128).copy()
        w = {"full": 0, "orbs_lin": 1, "nonlin": 2, "tdci": 3}[which]
        lib().orc_integrate_rk(self.h, C.c_int(0 if integrator == "euler" else 1), C.c_int(w), C.c_int(int(imag)),
                               _p(s), _d(t0), _d(t1))
        return s

    def metric_weights(self):
        """SIL metric: 1 on the coefficients, grid weights on every orbital point."""
        return np.concatenate([np.ones(self.nC), np.tile(self.w, self.nOS)])

    def sil(self, state, t0, t1, krylov_dim, tol=0.0, max_restarts=0, metric=None, which="orbs_lin"):
        s = np.ascontiguousarray(state, dtype=np.complex128).copy()
        w = {"full": 0, "orbs_lin": 1, "nonlin": 2, "tdci": 3}[which]
        m = None if metric is None else np.ascontiguousarray(metric, dtype=np.float64)
        lib().orc_integrate_sil(self.h, C.c_int(w), _p(s), _d(t0), _d(t1), C.c_int(krylov_dim), _d(tol),
                                C.c_int(max_restarts), _p(m))
        return s

    def propagate_split2(self, state, t0, t1, krylov_dim=0, tol=0.0, max_restarts=0, metric=None):
        s = np.ascontiguousarray(state, dtype=np.complex128).copy()
        m = None if metric is None else np.ascontiguousarray(metric, dtype=np.float64)
        lib().orc_propagate_split2(self.h, _p(s), _d(t0), _d(t1), C.c_int(krylov_dim), _d(tol),
                                   C.c_int(max_restarts), _p(m))
        return s

    def relax(self, state, dt, n_inner, conv_thresh, max_outer=100000):
        s = np.ascontiguousarray(state, dtype=np.complex128).copy()
        nout = C.c_int(0)
        e = lib().orc_relax(self.h, _p(s), _d(dt), C.c_int(n_inner), _d(conv_thresh), C.c_int(max_outer),
                            C.byref(nout))
        return e, s, nout.value


def gll(n, a=-1.0, b=1.0):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gll(C.c_int(n), _d(a), _d(b), _p(x), _p(w))
    return x, w


def eig_herm(A):
    A = np.asfortranarray(A, dtype=np.complex128)
    n = A.shape[0]
    ev = np.zeros(n)
    U = np.zeros((n, n), dtype=np.complex128, order="F")
    lib().orc_eig_herm(C.c_int(n), _p(A), _p(ev), _p(U))
    return ev, U


def eig_sym(A):
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    ev = np.zeros(n)
    U = np.zeros((n, n), order="F")
    lib().orc_eig_sym(C.c_int(n), _p(A), _p(ev), _p(U))
    return ev, U
