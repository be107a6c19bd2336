"""CPU: the field helpers that are host index and neighbour work (interpolate_field, apply_neumann_conditions,
cartesian_gradient_vec, enforce_cartesian_gradient_neumann) against the reference's own outputs
(tests/golden/fields_helpers.npz, made by make_golden.py), including the reference's unit test of
interpolate_field (updes/tests/test_interpolation.py)."""
import os

import numpy as np
import pytest

import cases as C
from updes_gb300 import SquareCloud
from updes_gb300 import fields as F

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "fields_helpers.npz"))


def _cloud(case, facets=None):
    return SquareCloud(Nx=case["Nx"], Ny=case["Ny"], facet_types=dict(facets or case["facets"]),
                       coords=C.grid_coords(dict(case, facets=facets or case["facets"])))


def test_interpolate_field_matches_the_reference():
    ic = C.FIELD_INTERP_CASE
    c1 = SquareCloud(Nx=ic["Nx"], Ny=ic["Ny"], facet_types=dict(ic["facets1"]))
    c2 = SquareCloud(Nx=ic["Nx"], Ny=ic["Ny"], facet_types=dict(ic["facets2"]))
    field = np.arange(c1.N)
    new = F.interpolate_field(field, c1, c2)
    assert np.array_equal(new, GOLD["interp_result"])
    # the reference's own assertion (test_interpolation.py): equal on the internal nodes
    assert np.allclose(field[:c1.Ni], new[:c2.Ni], atol=1e-12)
    # and every value arrives at the node with the same original id
    back = F.interpolate_field(new, c2, c1)
    assert np.array_equal(back, field)


def test_interpolate_field_refuses_clouds_of_different_sizes():
    c1 = SquareCloud(Nx=5, Ny=5, facet_types=dict(North="d", South="d", East="d", West="d"))
    c2 = SquareCloud(Nx=5, Ny=6, facet_types=dict(North="d", South="d", East="d", West="d"))
    with pytest.raises(AssertionError):
        F.interpolate_field(np.arange(c1.N), c1, c2)


def test_grid_finite_differences_match_the_reference():
    fd = C.FIELD_FD_CASE
    cloud = _cloud(fd)
    assert np.array_equal(cloud.sorted_nodes, GOLD["fd_sorted_nodes"])
    f = GOLD["fd_field"]
    bcs = {k: None for k in fd["facets"]}
    assert np.allclose(F.apply_neumann_conditions(f, bcs, cloud), GOLD["fd_neumann"], rtol=0, atol=1e-15)
    grads = F.cartesian_gradient_vec(range(cloud.N), f, cloud)
    assert np.allclose(grads, GOLD["fd_cartesian_gradient"], rtol=1e-13, atol=1e-13)
    enf = F.enforce_cartesian_gradient_neumann(f, grads, bcs, cloud)
    assert np.allclose(enf, GOLD["fd_enforced"], rtol=1e-13, atol=1e-13)
    # the Neumann rows changed, nothing else did
    nm = np.concatenate([cloud.facet_nodes[k] for k, t in fd["facets"].items() if t == "n"])
    other = np.setdiff1d(np.arange(cloud.N), nm)
    assert np.array_equal(enf[other], grads[other])


def test_small_helpers():
    a = np.arange(6.0).reshape(3, 2)
    b = np.ones((3, 2))
    assert np.array_equal(F.dot_vec(a, b), a.sum(axis=1))
    J = np.arange(12.0).reshape(3, 2, 2)
    assert np.array_equal(F.dot_mat(J, b), J.sum(axis=2))
    cl = SquareCloud(Nx=6, Ny=5, facet_types=dict(North="pn", South="pn", East="d", West="r"))
    bcs = {"North": np.ones(len(cl.facet_nodes["North"])), "South": 3.0, "East": 1.0,
           "West": (2.0, lambda x: 0.5 + x[1])}
    z = F.zerofy_periodic_cond(dict(bcs), cl)
    assert np.array_equal(z["North"], np.zeros(len(cl.facet_nodes["North"])))
    robin, vals = F.duplicate_robin_coeffs(bcs, cl)
    assert vals["West"] == 2.0 and vals["East"] == 1.0
    W = np.asarray(cl.facet_nodes["West"])
    assert sorted(robin) == sorted(int(i) for i in W)
    assert np.allclose([robin[int(i)] for i in W], 0.5 + cl.sorted_nodes[W, 1])
    # the solver's own Robin rows use the same coefficients
    from updes_gb300.operators import _bc_values_and_betas
    _, robin_solver = _bc_values_and_betas(bcs, cl, True)
    assert robin_solver == robin


def test_grid_finite_differences_on_local_supports_match_the_reference():
    fd = C.FIELD_FD_CASE
    cloud = SquareCloud(Nx=fd["Nx"], Ny=fd["Ny"], facet_types=dict(fd["facets"]), coords=C.grid_coords(fd),
                        support_size=C.FIELD_FD_SUPPORT)
    f = GOLD["fd_field"]
    bcs = {k: None for k in fd["facets"]}
    assert np.allclose(F.apply_neumann_conditions(f, bcs, cloud), GOLD["fdl_neumann"], rtol=0, atol=1e-15)
    grads = F.cartesian_gradient_vec(range(cloud.N), f, cloud)
    assert np.allclose(grads, GOLD["fdl_cartesian_gradient"], rtol=1e-13, atol=1e-13)
    assert np.allclose(F.enforce_cartesian_gradient_neumann(f, grads, bcs, cloud), GOLD["fdl_enforced"],
                       rtol=1e-13, atol=1e-13)
