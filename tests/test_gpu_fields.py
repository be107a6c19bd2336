"""GPU: the RBF field helpers (integrate_field, gradient_vals_vec, laplacian_vals_vec) against the reference's
outputs on its own integral test problem (updes/tests/test_integrals.py) and a jittered, non-square variant
(tests/golden/fields_helpers.npz).

* integrate_field of the reference's coefficients equals the reference's integral to 1e-12 (the same
  function evaluated at the same points, the reference's quadrature quirks included);
* from the product's own interpolation solve, the integral agrees to 1e-8 and passes the reference test's
  own bound (|integral - pi/12| < 0.1);
* gradients and Laplacians of the nodal field at seven points agree to 1e-6 of their scale: the r^11,
  degree-3 interpolation matrix is ill-conditioned, so two FP64 solvers' coefficients differ well above
  rounding while the interpolant they define does not.
"""
import os
from functools import partial

import numpy as np
import pytest

import cases as C
import updes_gb300 as U
from updes_gb300 import fields as F

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "fields_helpers.npz"))


def _setup(name):
    fc = C.FIELD_INTEGRAL_CASES[name]
    cloud = U.SquareCloud(Nx=fc["Nx"], Ny=fc["Ny"], facet_types=dict(fc["facets"]), coords=C.grid_coords(fc))
    assert np.array_equal(cloud.sorted_nodes, GOLD[f"{name}_sorted_nodes"])
    return fc, cloud, partial(U.polyharmonic, a=int(fc["rbf"][1]))


@pytest.mark.parametrize("name", list(C.FIELD_INTEGRAL_CASES))
def test_integrate_field_matches_the_reference(name):
    fc, cloud, rbf = _setup(name)
    ref = float(GOLD[f"{name}_integral"])
    got = F.integrate_field(GOLD[f"{name}_coeffs"], cloud, rbf, fc["max_degree"])
    assert abs(got - ref) <= 1e-12 * abs(ref), (got, ref)
    coeffs = U.compute_coefficients(C.field_s(cloud.sorted_nodes), cloud, rbf, fc["max_degree"])
    own = F.integrate_field(coeffs, cloud, rbf, fc["max_degree"])
    print(f"{name}: reference {ref:.15f}, from its coefficients {got:.15f}, own solve {own:.15f}")
    assert abs(own - ref) <= 1e-8 * abs(ref), (own, ref)
    assert abs(own - np.pi / 12) < 1e-1  # updes/tests/test_integrals.py


@pytest.mark.parametrize("name", list(C.FIELD_INTEGRAL_CASES))
def test_gradient_and_laplacian_of_nodal_values_match_the_reference(name):
    fc, cloud, rbf = _setup(name)
    s = C.field_s(cloud.sorted_nodes)
    g = F.gradient_vals_vec(C.FIELD_EVAL_POINTS, s, cloud, rbf, fc["max_degree"])
    lap = F.laplacian_vals_vec(C.FIELD_EVAL_POINTS, s, cloud, rbf, fc["max_degree"])
    gref, lref = GOLD[f"{name}_gradient_vals"], GOLD[f"{name}_laplacian_vals"]
    eg = np.max(np.abs(g - gref)) / np.max(np.abs(gref))
    el = np.max(np.abs(lap - lref)) / np.max(np.abs(lref))
    print(f"{name}: gradient {eg:.1e}, laplacian {el:.1e}")
    assert eg <= 1e-6 and el <= 1e-6
    one = F.gradient_vals(C.FIELD_EVAL_POINTS[0], s, cloud, rbf, fc["max_degree"])
    assert np.allclose(one, g[0], rtol=1e-12, atol=1e-12)
    one_l = F.laplacian_vals(C.FIELD_EVAL_POINTS[0], s, cloud, rbf, fc["max_degree"])
    assert abs(one_l - lap[0]) <= 1e-12 * max(1.0, abs(lap[0]))


def test_divergence_vec_is_the_sum_of_the_columns_gradients():
    name = "integral_12x9_jitter"
    fc, cloud, rbf = _setup(name)
    c = GOLD[f"{name}_coeffs"]
    c2 = np.stack([c, 2.0 * c], axis=-1)
    d = F.divergence_vec(C.FIELD_EVAL_POINTS, c2, cloud.sorted_nodes, rbf)
    g = U.gradient_vec(C.FIELD_EVAL_POINTS, c, cloud.sorted_nodes, rbf)
    assert np.allclose(d, g[:, 0] + 2.0 * g[:, 1], rtol=1e-13, atol=1e-13)
