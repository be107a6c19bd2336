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


def _product_cloud_from_fixture(g):
    """A product Cloud holding the reference's GmshCloud of its mesh fixture (stored arrays)."""
    import json

    from updes_gb300.cloud import Cloud
    facets = json.loads(str(g["facets"]))
    cl = Cloud(facet_types=facets)
    cl.N, cl.Ni, cl.Nd, cl.Nn, cl.Nr = (int(v) for v in g["counts"])
    cl.Np = []
    cl.sorted_nodes = np.ascontiguousarray(g["sorted_nodes"])
    cl.facet_nodes = {f: list(v) for f, v in json.loads(str(g["facet_nodes"])).items()}
    cl.node_types = {int(k): v for k, v in json.loads(str(g["node_types"])).items()}
    son = g["sorted_outward_normals"]
    cl.normals_by_node = np.zeros((cl.N, 2))
    cl.normals_by_node[cl.Ni + cl.Nd:cl.Ni + cl.Nd + son.shape[0]] = son
    cl.sorted_outward_normals = son
    cl.outward_normals = {cl.Ni + cl.Nd + k: son[k] for k in range(son.shape[0])}
    return cl


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_reference_unit_test_on_its_mesh_fixture(precision):
    """The reference's own unit test (updes/tests/test_operators.py:26-103) on the GPU: its GmshCloud of
    updes/tests/data/mesh.msh (stored by the fixture generator, which checked that this package's GmshCloud
    reads the file into the same cloud), every facet Neumann, Gaussian eps = 10, degree 1, operator
    nodal_value, rhs 12.  As there, the gradient and the divergence of the solution field at the nodes must
    be below 1e-2; the interior vals must equal the reference's (12) to 1e-8.  The boundary vals are not
    compared: that block of the system is numerically singular on this mesh, and the reference's own
    values there (+-1.5e4) differ from any other FP64 solver's by O(1)."""
    g = np.load(os.path.join(HERE, "ref_test_operators_mesh.npz"))
    cl = _product_cloud_from_fixture(g)
    rbf = partial(U.gaussian, eps=10.0)
    op = lambda x, center, rbf, monomial, fields: U.nodal_value(x, center, rbf, monomial)
    rhs = lambda x, centers, rbf, fields: 12.0 + 0.0 * x[0]
    bcs = {f: (lambda c: 0.0 * c[0]) for f in cl.facet_types}
    sol = U.pde_solver(op, rhs, cl, bcs, rbf, 1, options=U.SolverOptions(precision=precision,
                                                                         reuse_factorization=False))
    Ni = cl.Ni
    assert np.linalg.norm(sol.vals[:Ni] - g["vals"][:Ni]) <= 1e-8 * np.linalg.norm(g["vals"][:Ni])
    grads = U.gradient_vec(cl.sorted_nodes, sol.coeffs, cl.sorted_nodes, rbf)
    divs = U.divergence(cl.sorted_nodes, np.stack([sol.coeffs, sol.coeffs], axis=-1), cl.sorted_nodes, rbf)
    assert np.abs(np.linalg.norm(grads, axis=-1)).max() <= 1e-2
    assert np.abs(divs).max() <= 1e-2
