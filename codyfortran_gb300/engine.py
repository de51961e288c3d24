"""Host-side mirror of the reference's hot-path interface over the C ABI.

One :class:`Engine` wraps one ``cgpu_ctx`` (include/cody_gpu.h).  Method names
follow the reference procedures they replace; arrays use the reference
layouts (Fortran order, complex128).  Errors raise :class:`CodyError` with the
library's message, the counterpart of the reference's ``error stop``.

The CUDA library is mandatory: if ``libcodygpu.so`` is missing or no GPU is
present, construction raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .spec import SystemSpec

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libcodygpu.so")

TD_FULL, TD_ORBS_LIN, TD_NONLIN, TD_TDCI = 0, 1, 2, 3
_WHICH = {"full": TD_FULL, "orbs_lin": TD_ORBS_LIN, "nonlin": TD_NONLIN, "tdci": TD_TDCI}

EXPORTED = [
    "cgpu_ctx_create", "cgpu_ctx_destroy", "cgpu_last_error", "cgpu_last_global_error", "cgpu_host_alloc",
    "cgpu_host_free", "cgpu_select_device", "cgpu_sizes", "cgpu_grid",
    "cgpu_configlist_tables", "cgpu_synchronize", "cgpu_launch_count", "cgpu_time_derivative",
    "cgpu_apply_single_body_op", "cgpu_fill_h1", "cgpu_fill_h2", "cgpu_apply_correlation_op", "cgpu_energy",
    "cgpu_ci_apply_h1_fill_rdm1", "cgpu_ci_apply_h2_fill_rdm2", "cgpu_project_coeffs", "cgpu_normalize_coeffs",
    "cgpu_project_orbs", "cgpu_orthonormalize_orbs", "cgpu_integrate_rk4", "cgpu_integrate_euler",
    "cgpu_integrate_sil", "cgpu_propagate_split2", "cgpu_state_upload", "cgpu_state_download",
    "cgpu_propagate_resident", "cgpu_energy_resident", "cgpu_tdci_set_orbitals", "cgpu_propagate_resident_timed",
    "cgpu_profile_begin", "cgpu_profile_end", "cgpu_weighted_gram_noalloc",
    "cgpu_batch_create", "cgpu_batch_destroy", "cgpu_batch_size", "cgpu_batch_sizes", "cgpu_batch_grid",
    "cgpu_batch_upload", "cgpu_batch_download", "cgpu_batch_propagate", "cgpu_batch_energies",
    "cgpu_batch_kernels_per_step", "cgpu_batch_launch_count", "cgpu_batch_shared_interactions", "cgpu_batch_profile_begin", "cgpu_batch_profile_end",
    "cgpu_tdci_adjoint", "cgpu_observables", "cgpu_relax", "cgpu_batch_observables", "cgpu_save_restart",
    "cgpu_load_restart", "cgpu_absorber_setup", "cgpu_absorber_apply", "cgpu_batch_absorber_setup",
    "cgpu_batch_save_restart", "cgpu_batch_load_restart",
    "cgpu_autotune", "cgpu_get_tiles", "cgpu_set_tiles", "cgpu_batch_autotune", "cgpu_batch_get_tiles",
    "cgpu_batch_set_tiles", "cgpu_sys_kinetic_multiply", "cgpu_sys_potential_fill", "cgpu_sys_potential_multiply",
    "cgpu_sys_interaction_src", "cgpu_sys_interaction_potential", "cgpu_sys_interaction_multiply",
    "cgpu_mc_adjoint_forward", "cgpu_mc_adjoint_backward",
]

TUNE_CACHED, TUNE_FORCE = 0, 1
DEFAULT_TILE_CACHE = os.path.join(PKG, "_build", "tile_cache.jsonl")
TILE_KEYS = ("W", "Z", "H2")

KERNELS = {"pair_potentials": 1, "correlation": 2, "h2": 3, "ci_apply": 4, "ci_rdm": 5, "onebody": 6, "lanczos": 7,
           "rdm_inverse": 8, "projectors": 9, "fold": 10, "vector": 11}


class CodyError(RuntimeError):
    pass


class CgpuDesc(C.Structure):
    _fields_ = [
        ("grid_kind", C.c_int), ("xmin", C.c_double), ("xmax", C.c_double), ("n_points", C.c_int),
        ("n_elements", C.c_int), ("n_locals", C.c_int), ("xmin_excluded", C.c_int), ("xmax_excluded", C.c_int),
        ("n_body_types", C.c_int), ("n_bodies", C.c_int * 4), ("n_orbs", C.c_int * 4),
        ("body_mass", C.c_double * 4), ("restricted", C.c_int), ("regularization", C.c_double),
        ("n_nuclei", C.c_int), ("nuc_position", C.c_double * 8), ("nuc_charge", C.c_double * 8),
        ("nuc_softening1", C.c_double * 8), ("nuc_softening2", C.c_double * 8), ("nuc_dampening", C.c_double * 8),
        ("has_interaction", C.c_int), ("int_strength", C.c_double), ("int_softening1", C.c_double),
        ("int_softening2", C.c_double), ("int_dampening", C.c_double), ("int_kind", C.c_int),
        ("laser_kind", C.c_int), ("laser_E0", C.c_double), ("laser_omega", C.c_double),
        ("laser_n_cycles", C.c_double), ("laser_cep", C.c_double), ("laser_t_start", C.c_double),
        ("field_samples", C.POINTER(C.c_double)), ("n_field_samples", C.c_int), ("field_dt", C.c_double),
        ("field_t0", C.c_double), ("method", C.c_int), ("precision", C.c_int), ("max_krylov", C.c_int),
        ("krylov_window", C.c_int),
    ]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libcodygpu.so (built by codyfortran_gb300.build); raise if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise CodyError(f"CUDA library not built: {path} (run codyfortran_gb300.build.build())")
    lib = C.CDLL(path)
    for name in EXPORTED:
        getattr(lib, name)  # AttributeError if a symbol is missing
    lib.cgpu_last_error.restype = C.c_char_p
    lib.cgpu_last_error.argtypes = [C.c_void_p]
    lib.cgpu_last_global_error.restype = C.c_char_p
    lib.cgpu_launch_count.restype = C.c_long
    lib.cgpu_launch_count.argtypes = [C.c_void_p, C.c_int]
    lib.cgpu_ctx_create.argtypes = [C.POINTER(CgpuDesc), C.POINTER(C.c_void_p)]
    lib.cgpu_batch_create.argtypes = [C.POINTER(CgpuDesc), C.c_int, C.POINTER(C.c_void_p)]
    lib.cgpu_batch_kernels_per_step.restype = C.c_long
    lib.cgpu_batch_kernels_per_step.argtypes = [C.c_void_p]
    lib.cgpu_batch_launch_count.restype = C.c_long
    lib.cgpu_batch_launch_count.argtypes = [C.c_void_p, C.c_int]
    lib.cgpu_batch_shared_interactions.restype = C.c_int
    lib.cgpu_batch_shared_interactions.argtypes = [C.c_void_p]
    lib.cgpu_host_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    lib.cgpu_host_free.argtypes = [C.c_void_p]
    lib.cgpu_save_restart.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    lib.cgpu_load_restart.argtypes = [C.c_void_p, C.c_char_p]
    lib.cgpu_batch_save_restart.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    lib.cgpu_batch_load_restart.argtypes = [C.c_void_p, C.c_char_p]
    for name in ("cgpu_autotune", "cgpu_batch_autotune"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int]
    for name in ("cgpu_get_tiles", "cgpu_set_tiles", "cgpu_batch_get_tiles", "cgpu_batch_set_tiles"):
        getattr(lib, name).argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    _lib = lib
    return lib


class _PinnedBlock:
    """Page-locked host block from cgpu_host_alloc, exposed to numpy through the
    array interface and released when the last array over it is gone."""

    def __init__(self, n, dtype):
        self._lib = load_library()
        dt = np.dtype(dtype)
        ptr = C.c_void_p()
        if self._lib.cgpu_host_alloc(C.c_size_t(max(1, int(n)) * dt.itemsize), C.byref(ptr)) != 0:
            raise CodyError(self._lib.cgpu_last_global_error().decode())
        self._ptr = ptr.value
        self.__array_interface__ = {"shape": (int(n),), "typestr": dt.str, "data": (self._ptr, False), "version": 3}

    def __del__(self):
        if getattr(self, "_ptr", None):
            self._lib.cgpu_host_free(C.c_void_p(self._ptr))
            self._ptr = None


def tiles_to_dict(t):
    """The 10-entry tile table as {"W": (bn, compact, splits), "Z": ..., "H2": ..., "lz_blocks": n}."""
    t = [int(v) for v in t]
    d = {k: tuple(t[3 * i:3 * i + 3]) for i, k in enumerate(TILE_KEYS)}
    d["lz_blocks"] = t[9]
    return d


def tiles_from_dict(d):
    t = []
    for k in TILE_KEYS:
        t.extend(int(v) for v in d[k])
    t.append(int(d["lz_blocks"]))
    return (C.c_int * 10)(*t)


class _Tunable:
    """Tile table and autotuner of a context (cgpu_autotune / cgpu_get_tiles /
    cgpu_set_tiles), shared by Engine and Batch."""

    _tune_fns = ("cgpu_autotune", "cgpu_get_tiles", "cgpu_set_tiles")

    def autotune(self, cache_path=DEFAULT_TILE_CACHE, force=False):
        """Time the tile candidates on the resident states and apply the
        fastest (or the cached entry of this shape); returns the report dict."""
        import json
        fn = getattr(self.lib, self._tune_fns[0])
        buf = C.create_string_buffer(65536)
        path = None if cache_path is None else str(cache_path).encode()
        if cache_path is not None:
            os.makedirs(os.path.dirname(os.path.abspath(str(cache_path))), exist_ok=True)
        self._check(fn(self.h, path, TUNE_FORCE if force else TUNE_CACHED, buf, len(buf)))
        return json.loads(buf.value.decode())

    def tiles(self):
        t = (C.c_int * 10)()
        self._check(getattr(self.lib, self._tune_fns[1])(self.h, t))
        return tiles_to_dict(t)

    def set_tiles(self, d):
        self._check(getattr(self.lib, self._tune_fns[2])(self.h, tiles_from_dict(d)))


def select_device(device):
    """The CUDA device of the contexts this process creates from now on (one
    process per GPU passes its local rank)."""
    lib = load_library()
    if lib.cgpu_select_device(int(device)) != 0:
        raise CodyError(lib.cgpu_last_global_error().decode())


def pinned_empty(n, dtype=np.complex128):
    """Uninitialised 1-D array of n elements in page-locked host memory: state
    buffers whose uploads and downloads run as direct DMA."""
    return np.asarray(_PinnedBlock(n, dtype))


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _d(v):
    return C.c_double(float(v))


def make_desc(spec: SystemSpec, precision: str = "fp64", max_krylov: int = 32, krylov_window: int = 0):
    d = CgpuDesc()
    d.grid_kind = 0 if spec.grid_kind == "const" else 1
    d.xmin, d.xmax = spec.xmin, spec.xmax
    d.n_points, d.n_elements, d.n_locals = spec.n_points, spec.n_elements, spec.n_locals
    d.xmin_excluded, d.xmax_excluded = int(spec.xmin_excluded), int(spec.xmax_excluded)
    d.n_body_types = spec.n_bt
    for b in range(spec.n_bt):
        d.n_bodies[b] = int(spec.n_bodies[b])
        d.n_orbs[b] = int(spec.n_orbs[b])
        d.body_mass[b] = float(spec.masses[b])
    d.restricted = int(spec.restricted)
    d.regularization = spec.reg_eps
    d.n_nuclei = len(spec.nuclei)
    for i, n in enumerate(spec.nuclei):
        d.nuc_position[i], d.nuc_charge[i] = n.position, n.charge
        d.nuc_softening1[i], d.nuc_softening2[i], d.nuc_dampening[i] = n.softening1, n.softening2, n.dampening
    d.has_interaction = int(spec.has_interaction)
    d.int_strength, d.int_softening1, d.int_softening2, d.int_dampening = (
        spec.int_strength, spec.int_s1, spec.int_s2, spec.int_damp)
    d.int_kind = 0 if spec.int_kind == "toeplitz" else 1
    L = spec.laser
    d.laser_kind = {"none": 0, "sin2": 1, "sampled": 2}[L.kind]
    d.laser_E0, d.laser_omega, d.laser_n_cycles, d.laser_cep, d.laser_t_start = L.E0, L.omega, L.n_cycles, L.cep, L.t_start
    keep = None
    if L.kind == "sampled":
        keep = np.ascontiguousarray(L.samples, dtype=np.float64)
        d.field_samples = keep.ctypes.data_as(C.POINTER(C.c_double))
        d.n_field_samples = len(keep)
        d.field_dt, d.field_t0 = L.sample_dt, L.sample_t0
    d.method = 1 if spec.method == "tdci" else 0
    d.precision = {"fp64": 0, "mixed": 1, "mixed6": 2, "mixed_fx": 3, "mixed_fx6": 4}[precision]
    d.max_krylov = max_krylov
    d.krylov_window = int(krylov_window)
    return d, keep


class Engine(_Tunable):
    """The GB300 MCTDHX/TDCI engine for one system (one cgpu_ctx, one CUDA stream)."""

    def __init__(self, spec: SystemSpec, precision: str = "fp64", max_krylov: int = 32, krylov_window: int = 0):
        self.lib = load_library()
        self.spec = spec
        desc, self._keep = make_desc(spec, precision, max_krylov, krylov_window)
        h = C.c_void_p()
        rc = self.lib.cgpu_ctx_create(C.byref(desc), C.byref(h))
        if rc != 0:
            raise CodyError(self.lib.cgpu_last_global_error().decode())
        self.h = h
        sz = (C.c_int * 6)()
        self.lib.cgpu_sizes(self.h, sz)
        self.nG, self.nO, self.nOS, self.nC, self.nBt, self.nS = list(sz)
        self.x = np.zeros(self.nG)
        self.w = np.zeros(self.nG)
        self.lib.cgpu_grid(self.h, _p(self.x), _p(self.w))

    def close(self):
        if getattr(self, "h", None):
            self.lib.cgpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise CodyError(self.lib.cgpu_last_error(self.h).decode())

    def launch_count(self, reset=False):
        return self.lib.cgpu_launch_count(self.h, int(reset))

    # ConfigList --------------------------------------------------------------
    def tables(self, bt, kind):
        n_conf, mc = C.c_int(), C.c_int()
        self._check(self.lib.cgpu_configlist_tables(self.h, bt, kind, C.byref(n_conf), C.byref(mc), None, None, None,
                                                    None, None))
        n, m = n_conf.value, mc.value
        codes = np.zeros(n, dtype=np.int64)
        ncon = np.zeros(n, dtype=np.int32)
        exc = np.zeros(max(m, 1) * n, dtype=np.int32)
        oc = np.zeros(max(m, 1) * n, dtype=np.int32)
        fac = np.zeros(max(m, 1) * n, dtype=np.float64)
        self._check(self.lib.cgpu_configlist_tables(self.h, bt, kind, None, None, _p(codes), _p(ncon), _p(exc),
                                                    _p(oc), _p(fac)))
        f = lambda a: a[: m * n].reshape(n, m).T
        return dict(codes=codes, n_connected=ncon, excited_c=f(exc), orb_code=f(oc), factor=f(fac))

    # arrays -------------------------------------------------------------------
    def _orbs(self, orbs):
        return np.asfortranarray(orbs, dtype=np.complex128)

    def _new_orbs(self):
        return np.zeros((self.nG, self.nOS), dtype=np.complex128, order="F")

    def _n4(self):
        n = self.nO
        return np.zeros((n, n, n, n), dtype=np.complex128, order="F")

    def _n2(self):
        return np.zeros((self.nO, self.nO), dtype=np.complex128, order="F")

    # Method / Method_Mb_OrbBased ---------------------------------------------
    def time_derivative(self, state, t, which="full"):
        """Method_TimeDerivative / TimeDerivativeOrbsLin / ...CoeffsPlusOrbsNonLin / Tdci."""
        s = np.ascontiguousarray(state, dtype=np.complex128)
        d = np.zeros_like(s)
        self._check(self.lib.cgpu_time_derivative(self.h, _WHICH[which], _p(d), _p(s), _d(t)))
        return d

    def apply_single_body_op(self, orbs, t, want_h1=False, d_orbs=None):
        o = self._orbs(orbs)
        d = self._new_orbs() if d_orbs is None else np.array(d_orbs, dtype=np.complex128, order="F", copy=True)
        h1 = self._n2() if want_h1 else None
        self._check(self.lib.cgpu_apply_single_body_op(self.h, _p(d), _p(o), _d(t), _p(h1)))
        return (d, h1) if want_h1 else d

    def fill_h1(self, orbs, t):
        o = self._orbs(orbs)
        h1 = self._n2()
        self._check(self.lib.cgpu_fill_h1(self.h, _p(h1), _p(o), _d(t)))
        return h1

    def fill_h2(self, orbs, t):
        o = self._orbs(orbs)
        h2 = self._n4()
        self._check(self.lib.cgpu_fill_h2(self.h, _p(h2), _p(o), _d(t)))
        return h2

    def apply_correlation_op(self, orbs, rdm1, rdm2, t, d_orbs=None):
        o = self._orbs(orbs)
        r1 = np.asfortranarray(rdm1, dtype=np.complex128)
        r2 = np.asfortranarray(rdm2, dtype=np.complex128)
        d = self._new_orbs() if d_orbs is None else np.array(d_orbs, dtype=np.complex128, order="F", copy=True)
        h2 = self._n4()
        self._check(self.lib.cgpu_apply_correlation_op(self.h, _p(d), _p(o), _p(r1), _p(r2), _d(t), _p(h2)))
        return d, h2

    def energy(self, state, t=0.0):
        """Method_GetEnergy."""
        s = np.ascontiguousarray(state, dtype=np.complex128)
        e = C.c_double()
        self._check(self.lib.cgpu_energy(self.h, _p(s), _d(t), C.byref(e)))
        return e.value

    # Sys* operators on one orbital ---------------------------------------------
    def _vec(self, a):
        return np.ascontiguousarray(a, dtype=np.complex128)

    def sys_kinetic_multiply(self, orb, t=0.0, bt=1):
        """SysKinetic_MultiplyWithKineticOp: T orb with the mass of body type bt (1-based)."""
        out = np.zeros(self.nG, dtype=np.complex128)
        self._check(self.lib.cgpu_sys_kinetic_multiply(self.h, _p(out), _p(self._vec(orb)), _d(t), int(bt)))
        return out

    def sys_potential_fill(self, t=0.0, bt=1):
        """SysPotential_FillExternalPotential: V(x) + E(t) x."""
        out = np.zeros(self.nG, dtype=np.complex128)
        self._check(self.lib.cgpu_sys_potential_fill(self.h, _p(out), _d(t), int(bt)))
        return out

    def sys_potential_multiply(self, potential, orb):
        out = np.zeros(self.nG, dtype=np.complex128)
        self._check(self.lib.cgpu_sys_potential_multiply(self.h, _p(out), _p(self._vec(potential)),
                                                         _p(self._vec(orb))))
        return out

    def sys_interaction_src(self, orb_conjg, orb):
        """SysInteraction_FillInteractionSrc: conj(orb_conjg) orb w."""
        out = np.zeros(self.nG, dtype=np.complex128)
        self._check(self.lib.cgpu_sys_interaction_src(self.h, _p(out), _p(self._vec(orb_conjg)), _p(self._vec(orb))))
        return out

    def sys_interaction_potential(self, src, t=0.0, bt1=1, bt2=1):
        """SysInteraction_FillInteractionPotential: sum_j K(x_i, x_j) src_j."""
        out = np.zeros(self.nG, dtype=np.complex128)
        self._check(self.lib.cgpu_sys_interaction_potential(self.h, _p(out), _p(self._vec(src)), _d(t), int(bt1),
                                                            int(bt2)))
        return out

    def sys_interaction_multiply(self, potential, orb):
        out = np.zeros(self.nG, dtype=np.complex128)
        self._check(self.lib.cgpu_sys_interaction_multiply(self.h, _p(out), _p(self._vec(potential)),
                                                           _p(self._vec(orb))))
        return out

    # Coeffs -------------------------------------------------------------------
    def rdm1(self, coeffs):
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        r = self._n2()
        self._check(self.lib.cgpu_ci_apply_h1_fill_rdm1(self.h, _p(c), _p(r), None, None))
        return r

    def rdm2(self, coeffs):
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        r = self._n4()
        self._check(self.lib.cgpu_ci_apply_h2_fill_rdm2(self.h, _p(c), _p(r), None, None))
        return r

    def apply_h1(self, coeffs, h1, d_coeffs=None):
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        h = np.asfortranarray(h1, dtype=np.complex128)
        d = np.zeros(self.nC, dtype=np.complex128) if d_coeffs is None else np.array(d_coeffs, dtype=np.complex128)
        self._check(self.lib.cgpu_ci_apply_h1_fill_rdm1(self.h, _p(c), None, _p(d), _p(h)))
        return d

    def apply_h2(self, coeffs, h2, d_coeffs=None):
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        h = np.asfortranarray(h2, dtype=np.complex128)
        d = np.zeros(self.nC, dtype=np.complex128) if d_coeffs is None else np.array(d_coeffs, dtype=np.complex128)
        self._check(self.lib.cgpu_ci_apply_h2_fill_rdm2(self.h, _p(c), None, _p(d), _p(h)))
        return d

    def project_coeffs(self, d_coeffs, coeffs):
        d = np.array(d_coeffs, dtype=np.complex128)
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        self._check(self.lib.cgpu_project_coeffs(self.h, _p(d), _p(c)))
        return d

    def normalize_coeffs(self, coeffs):
        c = np.array(coeffs, dtype=np.complex128)
        self._check(self.lib.cgpu_normalize_coeffs(self.h, _p(c)))
        return c

    # Orbs ---------------------------------------------------------------------
    def project_orbs(self, d_orbs, orbs):
        d = np.array(d_orbs, dtype=np.complex128, order="F", copy=True)
        o = self._orbs(orbs)
        self._check(self.lib.cgpu_project_orbs(self.h, _p(d), _p(o)))
        return d

    def orthonormalize(self, orbs):
        o = np.array(orbs, dtype=np.complex128, order="F", copy=True)
        self._check(self.lib.cgpu_orthonormalize_orbs(self.h, _p(o)))
        return o

    # integrators / propagator -------------------------------------------------
    def metric_weights(self):
        return np.concatenate([np.ones(self.nC), np.tile(self.w, self.nOS)])

    def rk(self, state, t0, t1, integrator="rk4", which="nonlin", imag=False):
        s = np.array(state, dtype=np.complex128)
        if integrator == "euler":
            self._check(self.lib.cgpu_integrate_euler(self.h, _WHICH[which], int(imag), _p(s), _d(t0), _d(t1)))
        else:
            self._check(self.lib.cgpu_integrate_rk4(self.h, _WHICH[which], _p(s), _d(t0), _d(t1)))
        return s

    def sil(self, state, t0, t1, krylov_dim, tol=0.0, max_restarts=0, metric=None, which="orbs_lin"):
        s = np.array(state, dtype=np.complex128)
        m = None if metric is None else np.ascontiguousarray(metric, dtype=np.float64)
        warn = C.c_int()
        self._check(self.lib.cgpu_integrate_sil(self.h, _WHICH[which], _p(s), _d(t0), _d(t1), krylov_dim, _d(tol),
                                                max_restarts, _p(m), C.byref(warn)))
        return s

    def propagate_split2(self, state, t0, t1, krylov_dim=0, tol=0.0, max_restarts=0, use_metric=False, out=None):
        """Propagator_Propagate for SplitStep Order2 (host state in, host state
        out); `out` (complex128, contiguous, may be `state` itself) receives the
        result in place."""
        if out is None:
            s = np.array(state, dtype=np.complex128)
        else:
            if out.dtype != np.complex128 or not out.flags.c_contiguous or out.size != self.nS:
                raise CodyError("propagate_split2: out must be a contiguous complex128 array of nS entries")
            s = out
            if s is not state:
                s[:] = state
        self._check(self.lib.cgpu_propagate_split2(self.h, _p(s), _d(t0), _d(t1), krylov_dim, _d(tol), max_restarts,
                                                   int(use_metric)))
        return s

    # resident state -----------------------------------------------------------
    def upload(self, state):
        s = np.ascontiguousarray(state, dtype=np.complex128)
        self._check(self.lib.cgpu_state_upload(self.h, _p(s)))

    def download(self):
        s = np.zeros(self.nS, dtype=np.complex128)
        self._check(self.lib.cgpu_state_download(self.h, _p(s)))
        return s

    def propagate_resident(self, t0, dt, n_steps, krylov_dim, use_metric=True, use_graph=False):
        self._check(self.lib.cgpu_propagate_resident(self.h, _d(t0), _d(dt), int(n_steps), int(krylov_dim),
                                                     int(use_metric), int(use_graph)))

    def propagate_resident_timed(self, t0, dt, n_steps, krylov_dim, use_metric=True, use_graph=False):
        """Steps on the resident state; returns the device time (ms) from CUDA events on the context stream."""
        ms = C.c_double()
        self._check(self.lib.cgpu_propagate_resident_timed(self.h, _d(t0), _d(dt), int(n_steps), int(krylov_dim),
                                                           int(use_metric), int(use_graph), C.byref(ms)))
        return ms.value

    def profile_begin(self, kernel):
        self._check(self.lib.cgpu_profile_begin(self.h, KERNELS[kernel] if isinstance(kernel, str) else int(kernel)))

    def profile_end(self):
        n, ms = C.c_long(), C.c_double()
        self._check(self.lib.cgpu_profile_end(self.h, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def energy_resident(self, t):
        e = C.c_double()
        self._check(self.lib.cgpu_energy_resident(self.h, _d(t), C.byref(e)))
        return e.value

    def synchronize(self):
        self._check(self.lib.cgpu_synchronize(self.h))

    def observables(self, t):
        """Resident state at time t: dict(energy, norm, dipole, occupations)."""
        out = np.zeros(3 + self.nOS)
        self._check(self.lib.cgpu_observables(self.h, _d(t), _p(out)))
        return dict(energy=out[0], norm=out[1], dipole=out[2], occupations=out[3:].copy())

    def absorber(self, onset, order, apply_each_step=False):
        self._check(self.lib.cgpu_absorber_setup(self.h, _d(onset), _d(order), int(apply_each_step)))

    def absorber_apply(self):
        self._check(self.lib.cgpu_absorber_apply(self.h))

    def save_restart(self, directory, with_rdm2=False):
        self._check(self.lib.cgpu_save_restart(self.h, str(directory).encode(), int(with_rdm2)))

    def load_restart(self, directory):
        self._check(self.lib.cgpu_load_restart(self.h, str(directory).encode()))

    def relax(self, state, dt, n_inner, conv_thresh, max_outer=100000):
        """Imaginary-time relaxation on the GPU; returns (energy, state, rounds)."""
        s = np.array(state, dtype=np.complex128)
        e, n = C.c_double(), C.c_int()
        self._check(self.lib.cgpu_relax(self.h, _p(s), _d(dt), int(n_inner), _d(conv_thresh), int(max_outer),
                                        C.byref(e), C.byref(n)))
        return e.value, s, n.value

    # TDCI ---------------------------------------------------------------------
    def tdci_set_orbitals(self, orbs):
        o = self._orbs(orbs)
        self._check(self.lib.cgpu_tdci_set_orbitals(self.h, _p(o)))

    def mc_adjoint_forward(self, state0, field, dt, krylov_dim=12, checkpoint=64, ref_state=None):
        """MCTDHF pulse objective J = 1 - |<ref|Psi_N>|^2 after len(field)
        Strang steps with E(t) = field[floor(t / dt)]; keeps checkpoints for
        mc_adjoint_backward.  Returns (J, overlap, final state)."""
        s0 = np.ascontiguousarray(state0, dtype=np.complex128)
        ref = None if ref_state is None else np.ascontiguousarray(ref_state, dtype=np.complex128)
        f = np.ascontiguousarray(field, dtype=np.float64)
        self._mc_field_len = len(f)
        J, ov = C.c_double(), (C.c_double * 2)()
        fin = np.zeros_like(s0)
        self._check(self.lib.cgpu_mc_adjoint_forward(self.h, _p(s0), _p(ref), _p(f), len(f), _d(dt), int(krylov_dim),
                                                     int(checkpoint), C.byref(J), ov, _p(fin)))
        return J.value, complex(ov[0], ov[1]), fin

    def mc_adjoint_backward(self):
        """dJ/dfield[n] for the last mc_adjoint_forward."""
        g = np.zeros(getattr(self, "_mc_field_len", 0))
        self._check(self.lib.cgpu_mc_adjoint_backward(self.h, _p(g)))
        return g

    def tdci_adjoint(self, c0, field, dt, checkpoint=64, gradient=True):
        """J = 1 - |<c0|C_N>|^2 after len(field) RK4 steps (field constant per
        step) and, with gradient, dJ/dfield from the adjoint sweep.
        Returns (J, overlap, C_N, grad or None)."""
        c0 = np.ascontiguousarray(c0, dtype=np.complex128)
        f = np.ascontiguousarray(field, dtype=np.float64)
        J, ov = C.c_double(), (C.c_double * 2)()
        cn = np.zeros(self.nC, dtype=np.complex128)
        g = np.zeros(len(f)) if gradient else None
        self._check(self.lib.cgpu_tdci_adjoint(self.h, _p(c0), _p(f), len(f), _d(dt), int(checkpoint), C.byref(J), ov,
                                               _p(cn), _p(g)))
        return J.value, complex(ov[0], ov[1]), cn, g


class BatchSystem:
    """Sizes and grid of one system of a Batch."""

    def __init__(self, spec, sizes, x, w):
        self.spec = spec
        self.nG, self.nO, self.nOS, self.nC, self.nBt, self.nS = sizes
        self.x, self.w = x, w


class Batch(_Tunable):
    """Independent systems of arbitrary sizes advanced together: every kernel
    of the step covers all systems in one launch, one CUDA-graph launch per
    time step (cgpu_batch_propagate)."""

    _tune_fns = ("cgpu_batch_autotune", "cgpu_batch_get_tiles", "cgpu_batch_set_tiles")

    def __init__(self, specs, precision: str = "fp64", max_krylov: int = 32, krylov_window: int = 0):
        self.lib = load_library()
        self.specs = list(specs)
        n = len(self.specs)
        descs = (CgpuDesc * n)()
        self._keep = []
        for i, sp in enumerate(self.specs):
            d, keep = make_desc(sp, precision, max_krylov, krylov_window)
            descs[i] = d
            self._keep.append(keep)
        h = C.c_void_p()
        rc = self.lib.cgpu_batch_create(descs, n, C.byref(h))
        if rc != 0:
            raise CodyError(self.lib.cgpu_last_global_error().decode())
        self.h = h
        self.systems = []
        for i, sp in enumerate(self.specs):
            sz = (C.c_int * 6)()
            self.lib.cgpu_batch_sizes(self.h, i, sz)
            x, w = np.zeros(sz[0]), np.zeros(sz[0])
            self.lib.cgpu_batch_grid(self.h, i, _p(x), _p(w))
            self.systems.append(BatchSystem(sp, list(sz), x, w))
        self.offsets = np.concatenate([[0], np.cumsum([s.nS for s in self.systems])]).astype(np.int64)

    def __len__(self):
        return len(self.systems)

    def close(self):
        if getattr(self, "h", None):
            self.lib.cgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise CodyError(self.lib.cgpu_last_global_error().decode())

    def pack(self, states):
        return np.ascontiguousarray(np.concatenate([np.asarray(s, dtype=np.complex128) for s in states]))

    def upload(self, states):
        """states: list of per-system state vectors, or one packed array."""
        buf = states if isinstance(states, np.ndarray) and states.ndim == 1 and states.size == self.offsets[-1] \
            else self.pack(states)
        buf = np.ascontiguousarray(buf, dtype=np.complex128)
        self._check(self.lib.cgpu_batch_upload(self.h, _p(buf)))

    def download_packed(self, out=None):
        buf = out if out is not None else np.zeros(int(self.offsets[-1]), dtype=np.complex128)
        self._check(self.lib.cgpu_batch_download(self.h, _p(buf)))
        return buf

    def download(self):
        buf = self.download_packed()
        return [buf[self.offsets[i]:self.offsets[i + 1]].copy() for i in range(len(self))]

    def propagate(self, t0, dt, n_steps, krylov_dim, use_metric=True):
        """n_steps fixed-order Strang steps of every system (start times t0,
        scalar or one per system); returns the device time in ms."""
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, dtype=np.float64), (len(self),)))
        ms = C.c_double()
        self._check(self.lib.cgpu_batch_propagate(self.h, _p(t), _d(dt), int(n_steps), int(krylov_dim),
                                                  int(use_metric), C.byref(ms)))
        return ms.value

    def save_restart(self, directory, with_rdm2=False):
        """Every trajectory's restart files under directory/trajNNNNN/."""
        self._check(self.lib.cgpu_batch_save_restart(self.h, str(directory).encode(), int(with_rdm2)))

    def load_restart(self, directory):
        self._check(self.lib.cgpu_batch_load_restart(self.h, str(directory).encode()))

    def observables(self, t):
        """(energy, norm, dipole, occupations[nOSmax]) arrays over the systems at times t."""
        tt = np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64), (len(self),)))
        nmax = max(s.nOS for s in self.systems)
        out = np.zeros((len(self), 3 + nmax))
        self._check(self.lib.cgpu_batch_observables(self.h, _p(tt), _p(out)))
        return out[:, 0], out[:, 1], out[:, 2], out[:, 3:]

    def energies(self, t):
        tt = np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64), (len(self),)))
        e = np.zeros(len(self))
        self._check(self.lib.cgpu_batch_energies(self.h, _p(tt), _p(e)))
        return e

    def shared_interactions(self):
        """Number of interaction matrices shared by the batch (fixed-point form), 0 if none."""
        return self.lib.cgpu_batch_shared_interactions(self.h)

    def kernels_per_step(self):
        return self.lib.cgpu_batch_kernels_per_step(self.h)

    def profile_begin(self, kernel):
        self._check(self.lib.cgpu_batch_profile_begin(self.h, KERNELS[kernel] if isinstance(kernel, str) else int(kernel)))

    def profile_end(self):
        n, ms = C.c_long(), C.c_double()
        self._check(self.lib.cgpu_batch_profile_end(self.h, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def launch_count(self, reset=False):
        return self.lib.cgpu_batch_launch_count(self.h, int(reset))
