"""GPU: pde_solver_jit on a GmshCloud (synthetic Gmsh 4.0.8 mesh with a curved Robin facet) against the
reference's pde_solver_jit on its own GmshCloud of the same file (golden vectors)."""
import os
from functools import partial

import numpy as np
import pytest

import cases as C
import updes_gb300 as U
from updes_gb300.cloud import GmshCloud

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-8)])
def test_solve_on_gmsh_cloud_matches_reference(precision, tol):
    g = np.load(os.path.join(HERE, "gmsh_dshape.npz"))
    case = C.GMSH_CASE
    cloud = GmshCloud(os.path.join(HERE, case["mesh"]), facet_types=dict(case["facets"]))
    rbf = partial(U.polyharmonic, a=int(case["rbf"][1]))
    op = lambda x, center, rbf, monomial, fields: U.nodal_laplacian(x, center, rbf, monomial)
    rhs = lambda x, centers, rbf, fields: C.FUNCS[case["rhs"]](np, x[0], x[1])
    fn = lambda name: (lambda c: C.FUNCS[name](np, c[0], c[1]))
    bcs = {f: (fn(v[0]), fn(v[1])) if isinstance(v, tuple) else fn(v) for f, v in case["bc"].items()}
    sol = U.pde_solver_jit(op, rhs, cloud, bcs, rbf, case["max_degree"],
                           options=U.SolverOptions(precision=precision))
    assert np.linalg.norm(sol.vals - g["vals"]) <= tol * np.linalg.norm(g["vals"])
