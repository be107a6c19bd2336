"""GPU: pde_multi_solver (Picard sweeps over pde_solver) against the reference's own pde_multi_solver
(golden vectors made by running the reference, updes/operators.py:686-771)."""
import os
from functools import partial

import numpy as np
import pytest

import cases as C
import updes_gb300 as U

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _system(case):
    coords = C.grid_coords(case)
    cloud = U.SquareCloud(Nx=case["Nx"], Ny=case["Ny"], facet_types=dict(case["facets"]), coords=coords)
    rbf = partial(U.polyharmonic, a=int(case["rbf"][1]))
    if case["kind"] == "grayscott":
        def dop(x, center=None, rbf=None, monomial=None, fields=None):
            return U.nodal_value(x, center, rbf, monomial)

        def rop_u(x, centers=None, rbf=None, fields=None):
            u, v = U.value(x, fields[:, 0], centers, rbf), U.value(x, fields[:, 1], centers, rbf)
            return C.GS_DU * U.laplacian(x, fields[:, 0], centers, rbf) - u * v ** 2 + C.GS_F * (1 - u)

        def rop_v(x, centers=None, rbf=None, fields=None):
            u, v = U.value(x, fields[:, 0], centers, rbf), U.value(x, fields[:, 1], centers, rbf)
            return C.GS_DV * U.laplacian(x, fields[:, 1], centers, rbf) + u * v ** 2 - (C.GS_F + C.GS_K) * v
    else:
        def dop(x, center=None, rbf=None, monomial=None, fields=None):
            g = U.nodal_gradient(x, center, rbf, monomial)
            return U.nodal_value(x, center, rbf, monomial) / C.BURGERS_DT + fields[0] * g[0] + fields[1] * g[1]

        def rop_u(x, centers=None, rbf=None, fields=None):
            return U.value(x, fields[:, 0], centers, rbf) / C.BURGERS_DT

        def rop_v(x, centers=None, rbf=None, fields=None):
            return U.value(x, fields[:, 1], centers, rbf) / C.BURGERS_DT
    zero = lambda c: 0.0 * c[0]
    bcs = {f: zero for f in case["facets"]}
    return cloud, rbf, [dop, dop], [rop_u, rop_v], [dict(bcs), dict(bcs)]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", list(C.MULTI_CASES))
def test_multi_solver_matches_reference(name, precision):
    g = np.load(os.path.join(HERE, f"{name}.npz"))
    case = C.MULTI_CASES[name]
    cloud, rbf, dops, rops, bcs = _system(case)
    assert np.array_equal(cloud.sorted_nodes, g["sorted_nodes"])
    u0, v0 = C.multi_initial(case, cloud.sorted_nodes)
    prev = [u0, v0]
    sols = U.pde_multi_solver(dops, rops, cloud, bcs, rbf, case["max_degree"], nb_iters=case["nb_iters"], tol=1e-10,
                              diff_args=[prev, prev], rhs_args=[prev, prev],
                              options=U.SolverOptions(precision=precision))
    tol = 1e-10 if precision == "fp64" else 1e-8
    for i in range(2):
        assert np.linalg.norm(sols[i].vals - g["vals"][i]) <= tol * np.linalg.norm(g["vals"][i])
    assert len(U.operators.LAST_MULTI_INFO["changes"]) == case["nb_iters"]


def test_multi_solver_rejects_mismatched_lists():
    """Checked on the host before any solve (no GPU needed)."""
    case = C.MULTI_CASES["multi_advect_9x9"]
    cloud, rbf, dops, rops, bcs = _system(case)
    with pytest.raises(AssertionError):
        U.pde_multi_solver(dops, rops[:1], cloud, bcs, rbf, 1, diff_args=[[0, 0], [0, 0]])
