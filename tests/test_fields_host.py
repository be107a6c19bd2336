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
