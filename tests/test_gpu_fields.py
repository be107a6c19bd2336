"""GPU: the RBF field helpers (integrate_field, gradient_vals_vec, laplacian_vals_vec, divergence_vec) on the
reference's own integral test problem (updes/tests/test_integrals.py: 12 x 12 Dirichlet grid, r^11, degree
3, s = x^2 / (1 + y^2)) and a jittered, non-square variant.

* integrate_field of the reference's own coefficients equals the reference's integral to 1e-12 (the same
  function at the same points, the reference's quadrature quirks included: tests/golden/fields_helpers.npz).
* With coefficients from the product's own interpolation solve, the integral and gradients agree to 1e-9,
  the Laplacians to 1e-8, with a NumPy evaluation of the FP64 LU solution: the interpolation matrix has a
  condition number of about 2e12, and FP64 LU solutions of it with every entry moved by an ulp spread by
  2e-13 (integral), 1.2e-11 (gradients) and 5.6e-10 (Laplacians).  The reference forms its coefficients as
  inv(A) @ [s; 0], which moves them further (on the uniform grid its integral is 7e-7 from the LU's, its
  gradients 6e-6 and Laplacians 1.5e-4 of their scale), so against the reference the bounds are 1e-5,
  1e-4 and 1e-3, and the reference test's own bound (|integral - pi/12| < 0.1) holds.
"""
import os
from functools import partial

import numpy as np
import pytest
import scipy.linalg as sl

import cases as C
import updes_gb300 as U
from updes_gb300 import fields as F

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "fields_helpers.npz"))
_EXPS = [(0, 0), (1, 0), (0, 1), (2, 0), (1, 1), (0, 2), (3, 0), (2, 1), (1, 2), (0, 3)]


def _setup(name):
    fc = C.FIELD_INTEGRAL_CASES[name]
    cloud = U.SquareCloud(Nx=fc["Nx"], Ny=fc["Ny"], facet_types=dict(fc["facets"]), coords=C.grid_coords(fc))
    assert np.array_equal(cloud.sorted_nodes, GOLD[f"{name}_sorted_nodes"])
    return fc, cloud, partial(U.polyharmonic, a=int(fc["rbf"][1]))


def _lu_field(cloud, fc):
    """Coefficients of s by an FP64 LU of A = [[Phi, P], [P^T, 0]] on the CPU, and (value, gradient,
    Laplacian) evaluators of the field they define (r^k closed forms, monomials of degree <= 3)."""
    X, k = cloud.sorted_nodes, 2 * int(fc["rbf"][1]) + 1
    M = {0: 1, 1: 3, 2: 6, 3: 10}[fc["max_degree"]]
    ex = _EXPS[:M]
    mono = lambda P: np.stack([P[:, 0] ** a * P[:, 1] ** b for a, b in ex], axis=1)
    r = np.linalg.norm(X[:, None] - X[None], axis=2)
    A = np.block([[r ** k, mono(X)], [mono(X).T, np.zeros((M, M))]])
    c = sl.lu_solve(sl.lu_factor(A), np.concatenate([C.field_s(X), np.zeros(M)]))
    lam, gam = c[:len(X)], c[len(X):]

    def value(P):
        rr = np.linalg.norm(P[:, None] - X[None], axis=2)
        return rr ** k @ lam + mono(P) @ gam

    def grad(P):
        d = P[:, None] - X[None]
        rr = np.linalg.norm(d, axis=2)
        g = np.einsum("pj,pjc->pc", k * rr ** (k - 2) * lam[None], d)
        dm = np.stack([np.stack([a * P[:, 0] ** max(a - 1, 0) * P[:, 1] ** b for a, b in ex], 1),
                       np.stack([b * P[:, 0] ** a * P[:, 1] ** max(b - 1, 0) for a, b in ex], 1)], -1)
        return g + np.einsum("pmc,m->pc", dm, gam)

    def lap(P):
        rr = np.linalg.norm(P[:, None] - X[None], axis=2)
        lm = np.stack([a * (a - 1) * P[:, 0] ** max(a - 2, 0) * P[:, 1] ** b +
                       b * (b - 1) * P[:, 0] ** a * P[:, 1] ** max(b - 2, 0) for a, b in ex], 1)
        return (k * k * rr ** (k - 2)) @ lam + lm @ gam

    return c, value, grad, lap


@pytest.mark.parametrize("name", list(C.FIELD_INTEGRAL_CASES))
def test_integrate_field(name):
    fc, cloud, rbf = _setup(name)
    ref = float(GOLD[f"{name}_integral"])
    got = F.integrate_field(GOLD[f"{name}_coeffs"], cloud, rbf, fc["max_degree"])
    assert abs(got - ref) <= 1e-12 * abs(ref), (got, ref)
    c_lu, value, _, _ = _lu_field(cloud, fc)
    orig = F.value_vec
    F.value_vec = lambda pts, field, centers, rbf: value(np.asarray(pts))
    try:
        want = F.integrate_field(c_lu, cloud, rbf, fc["max_degree"])
    finally:
        F.value_vec = orig
    coeffs = U.compute_coefficients(C.field_s(cloud.sorted_nodes), cloud, rbf, fc["max_degree"])
    own = F.integrate_field(coeffs, cloud, rbf, fc["max_degree"])
    print(f"{name}: reference {ref:.15f}, FP64 LU {want:.15f}, own solve {own:.15f}")
    assert abs(own - want) <= 1e-9 * abs(want), (own, want)
    assert abs(own - ref) <= 1e-5 * abs(ref), (own, ref)
    assert abs(own - np.pi / 12) < 1e-1  # updes/tests/test_integrals.py


@pytest.mark.parametrize("name", list(C.FIELD_INTEGRAL_CASES))
def test_gradient_and_laplacian_of_nodal_values(name):
    fc, cloud, rbf = _setup(name)
    s = C.field_s(cloud.sorted_nodes)
    P = C.FIELD_EVAL_POINTS
    g = F.gradient_vals_vec(P, s, cloud, rbf, fc["max_degree"])
    lap = F.laplacian_vals_vec(P, s, cloud, rbf, fc["max_degree"])
    _, _, grad, lapf = _lu_field(cloud, fc)
    gw, lw = grad(P), lapf(P)
    gref, lref = GOLD[f"{name}_gradient_vals"], GOLD[f"{name}_laplacian_vals"]
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    print(f"{name}: vs FP64 LU gradient {rel(g, gw):.1e} laplacian {rel(lap, lw):.1e}; "
          f"vs reference {rel(g, gref):.1e} {rel(lap, lref):.1e}")
    assert rel(g, gw) <= 1e-9 and rel(lap, lw) <= 1e-8
    assert rel(g, gref) <= 1e-4 and rel(lap, lref) <= 1e-3
    one = F.gradient_vals(P[0], s, cloud, rbf, fc["max_degree"])
    assert np.allclose(one, g[0], rtol=1e-12, atol=1e-12)
    one_l = F.laplacian_vals(P[0], s, cloud, rbf, fc["max_degree"])
    assert abs(one_l - lap[0]) <= 1e-12 * max(1.0, abs(lap[0]))


def test_divergence_vec_is_the_sum_of_the_columns_gradients():
    name = "integral_12x9_jitter"
    fc, cloud, rbf = _setup(name)
    c = GOLD[f"{name}_coeffs"]
    c2 = np.stack([c, 2.0 * c], axis=-1)
    d = F.divergence_vec(C.FIELD_EVAL_POINTS, c2, cloud.sorted_nodes, rbf)
    g = U.gradient_vec(C.FIELD_EVAL_POINTS, c, cloud.sorted_nodes, rbf)
    assert np.allclose(d, g[:, 0] + 2.0 * g[:, 1], rtol=1e-13, atol=1e-13)
