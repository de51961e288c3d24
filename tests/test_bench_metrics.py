"""The reporting helpers of bench.py on the CPU: the orbital-span defect of
the mixed-precision deviation report and the slice-product count behind the
roofline's issued rate."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _orthonormal(rng, nG, n, w):
    a = rng.normal(size=(nG, n)) + 1j * rng.normal(size=(nG, n))
    q, _ = np.linalg.qr(a * np.sqrt(w)[:, None])  # orthonormal in the weighted metric
    return q / np.sqrt(w)[:, None]


def _state(C, phi):
    return np.concatenate([C, phi.T.reshape(-1)])  # [C | phi(nG, n) column-major]


def test_span_defect_zero_for_the_same_span_and_invariant_under_rotation():
    rng = np.random.default_rng(3)
    nG, n, nC = 60, 4, 6
    w = rng.uniform(0.5, 1.5, nG)
    phi = _orthonormal(rng, nG, n, w)
    C = rng.normal(size=nC) + 0j
    u, _ = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    a, b = _state(C, phi), _state(C, phi @ u)
    assert bench.orbital_span_defect(a, a, nC, nG, n, w) < 1e-13
    assert bench.orbital_span_defect(a, b, nC, nG, n, w) < 1e-13


def test_span_defect_second_order_in_a_rotation_out_of_the_span():
    rng = np.random.default_rng(4)
    nG, n, nC = 80, 3, 5
    w = rng.uniform(0.5, 1.5, nG)
    q = _orthonormal(rng, nG, n + 1, w)
    phi, extra = q[:, :n], q[:, n]
    C = np.ones(nC, dtype=complex)
    out = []
    for eps in (1e-3, 2e-3):
        moved = phi.copy()
        moved[:, 0] = np.cos(eps) * phi[:, 0] + np.sin(eps) * extra  # still orthonormal
        out.append(bench.orbital_span_defect(_state(C, phi), _state(C, moved), nC, nG, n, w))
    assert abs(out[0] - 0.5e-6) < 1e-9  # 1 - cos(eps) ~ eps^2 / 2
    assert abs(out[1] / out[0] - 4.0) < 1e-3


def test_slice_products_per_algorithmic_product():
    class Sys:
        def __init__(self, nG):
            self.nG = nG
    long_grid, short_grid = [Sys(501), Sys(2001)], [Sys(200)]
    assert bench.fx_grid_products("mixed_fx6", long_grid) == 21  # 6-bit digits, 6 slices
    assert bench.fx_grid_products("mixed_fx", long_grid) == 15   # 6-bit digits, 5 slices
    assert bench.fx_grid_products("mixed_fx6", short_grid) == 15  # 8-bit digits, 5 slices
