"""The no-allocation Gram entry point against the existing FillH1 entry point.

cgpu_weighted_gram_noalloc serves callers that cannot call cudaMalloc: it
takes the caller's device buffers and keeps its partial sums in a fixed
array inside the library.  For one body type, FillH1's h1 is exactly the
weighted Gram matrix <phi_i | h phi_j>, so the new entry point, fed with
the orbitals and the existing ApplySingleBodyOp output, must reproduce
cgpu_fill_h1.  Two calls in a row (different times, hence different inputs)
show that nothing left in the shared array from the first call leaks into
the second.

This file is collected last.  It passes run alone in a fresh process and
after the rest of the suite.
"""
import ctypes as C
import ctypes.util
import os

import numpy as np
import pytest

from codyfortran_gb300 import init as I
from codyfortran_gb300 import spec as S

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _cudart():
    cands = ["/usr/local/cuda/lib64/libcudart.so", ctypes.util.find_library("cudart")]
    cands += [f"/usr/local/cuda/lib64/libcudart.so.{v}" for v in (13, 12)]
    for p in cands:
        if p and os.path.exists(p):
            return C.CDLL(p)
    if ctypes.util.find_library("cudart"):
        return C.CDLL(ctypes.util.find_library("cudart"))
    pytest.fail("libcudart not found")


class DeviceBuffer:
    """Caller-owned device memory (the test harness may allocate; the entry point may not)."""

    def __init__(self, rt, host):
        self.rt = rt
        self.nbytes = host.nbytes
        self.ptr = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), C.c_size_t(self.nbytes)) == 0
        self.upload(host)

    def upload(self, host):
        assert self.rt.cudaMemcpy(self.ptr, host.ctypes.data_as(C.c_void_p), C.c_size_t(self.nbytes), 1) == 0

    def download(self, host):
        assert self.rt.cudaMemcpy(host.ctypes.data_as(C.c_void_p), self.ptr, C.c_size_t(self.nbytes), 2) == 0

    def free(self):
        self.rt.cudaFree(self.ptr)


def _system():
    return S.SystemSpec(
        grid_kind="fedvr", xmin=-16.0, xmax=16.0, n_elements=16, n_locals=8,
        n_bodies=(3,), n_orbs=(6,), masses=(1.0,), stats="f", restricted=False,
        nuclei=[S.Nucleus(-2.0, 1.5, 1.0, 0.0, 0.0), S.Nucleus(2.0, 1.5, 1.0, 0.0, 0.1)],
        int_kind="dense", laser=S.sin2_pulse(0.05, omega=0.3, n_cycles=2.0, cep=0.4))


def test_noalloc_gram_matches_fill_h1_on_two_calls():
    from codyfortran_gb300 import build
    from codyfortran_gb300.engine import Engine
    build.build()
    sp = _system()
    e = Engine(sp)
    lib = e.lib
    rt = _cudart()
    orbs = I.seeded_gaussian_orbitals(sp, e.x, e.w, 3)
    n, nG = e.nOS, e.nG
    a = DeviceBuffer(rt, np.asfortranarray(orbs))
    b = DeviceBuffer(rt, np.zeros((nG, n), dtype=np.complex128, order="F"))
    w = DeviceBuffer(rt, np.ascontiguousarray(e.w))
    g = DeviceBuffer(rt, np.zeros((n, n), dtype=np.complex128, order="F"))
    try:
        for t in (0.7, 31.0):
            h1 = e.fill_h1(orbs, t)                         # existing entry point
            h_orbs = e.apply_single_body_op(orbs, t)        # existing entry point: h phi
            b.upload(np.asfortranarray(h_orbs))
            rc = lib.cgpu_weighted_gram_noalloc(a.ptr, b.ptr, w.ptr, nG, n, g.ptr, None)
            assert rc == 0, lib.cgpu_last_global_error().decode()
            assert rt.cudaDeviceSynchronize() == 0
            out = np.zeros((n, n), dtype=np.complex128, order="F")
            g.download(out)
            err = np.linalg.norm(out - h1) / np.linalg.norm(h1)
            assert err < TOL, (t, err)
        # sizes beyond the fixed scratch are refused with a clear message
        rc = lib.cgpu_weighted_gram_noalloc(a.ptr, b.ptr, w.ptr, nG, 33, g.ptr, None)
        assert rc == 1 and b"1..32" in lib.cgpu_last_global_error()
    finally:
        for buf in (a, b, w, g):
            buf.free()
        e.close()


def test_noalloc_gram_wide_and_long_against_numpy():
    """Caller-owned random buffers at the edges of the fixed scratch: 17 and 32
    columns (every accumulator slot of a thread in use), a grid longer than the
    64 blocks x 32 points one pass covers (blocks loop), then a short grid on
    the same buffers (fewer blocks than the call before), each against numpy."""
    from codyfortran_gb300 import build
    from codyfortran_gb300.engine import load_library
    build.build()
    lib = load_library()
    rt = _cudart()
    rng = np.random.default_rng(17)
    for n in (17, 32):
        nG = 5000
        A = np.asfortranarray(rng.normal(size=(nG, n)) + 1j * rng.normal(size=(nG, n)))
        B = np.asfortranarray(rng.normal(size=(nG, n)) + 1j * rng.normal(size=(nG, n)))
        w = rng.uniform(0.1, 2.0, size=nG)
        a, b, wd = DeviceBuffer(rt, A), DeviceBuffer(rt, B), DeviceBuffer(rt, w)
        g = DeviceBuffer(rt, np.zeros((n, n), dtype=np.complex128, order="F"))
        try:
            for n_grid in (nG, 300):
                rc = lib.cgpu_weighted_gram_noalloc(a.ptr, b.ptr, wd.ptr, n_grid, n, g.ptr, None)
                assert rc == 0, lib.cgpu_last_global_error().decode()
                assert rt.cudaDeviceSynchronize() == 0
                out = np.zeros((n, n), dtype=np.complex128, order="F")
                g.download(out)
                # the first n_grid rows of each column (column stride n_grid)
                Ak = A.ravel(order="F")[: n_grid * n].reshape(n, n_grid).T
                Bk = B.ravel(order="F")[: n_grid * n].reshape(n, n_grid).T
                ref = Ak.conj().T @ (w[:n_grid, None] * Bk)
                err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
                assert err < TOL, (n, n_grid, err)
        finally:
            for buf in (a, b, wd, g):
                buf.free()
