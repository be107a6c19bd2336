"""CPU: GmshCloud (updes/cloud.py:520-734) against the reference's own GmshCloud on a synthetic Gmsh 4.0.8
mesh (tests/golden/make_msh.py), and the oracle's solve on that cloud against the reference's pde_solver_jit."""
import json
import os

import numpy as np
import pytest

import cases as C
from oracle import updes_np as O
from updes_gb300.cloud import GmshCloud

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden():
    return np.load(os.path.join(HERE, "gmsh_dshape.npz"))


def _cloud():
    case = C.GMSH_CASE
    return GmshCloud(os.path.join(HERE, case["mesh"]), facet_types=dict(case["facets"]))


def test_gmsh_cloud_matches_reference():
    g = _golden()
    cl = _cloud()
    assert [cl.N, cl.Ni, cl.Nd, cl.Nn, cl.Nr] == g["counts"].tolist()
    assert np.array_equal(cl.sorted_nodes, g["sorted_nodes"])
    assert cl.facet_nodes == json.loads(str(g["facet_nodes"]))
    assert {str(k): v for k, v in cl.node_types.items()} == json.loads(str(g["node_types"]))
    assert {str(k): v for k, v in cl.renumbering_map.items()} == json.loads(str(g["renumbering"]))
    assert cl.sorted_outward_normals.shape == g["sorted_outward_normals"].shape
    assert np.allclose(cl.sorted_outward_normals, g["sorted_outward_normals"], rtol=0, atol=1e-12)


def test_oracle_solve_on_gmsh_cloud_matches_reference():
    """The reference's cloud (from the golden file) through the oracle's faithful solve order."""
    g = _golden()
    case = C.GMSH_CASE
    N, Ni, Nd, Nn, Nr = g["counts"].tolist()
    X = g["sorted_nodes"]
    son = g["sorted_outward_normals"]
    facet_nodes = {f: list(v) for f, v in json.loads(str(g["facet_nodes"])).items()}
    normals = {Ni + Nd + k: son[k] for k in range(son.shape[0])}
    cl = O.Cloud(Nx=0, Ny=0, facet_types=dict(case["facets"]), N=N, Ni=Ni, Nd=Nd, Nn=Nn, Nr=Nr, Np=[],
                 sorted_nodes=X, node_types={int(k): v for k, v in json.loads(str(g["node_types"])).items()},
                 facet_nodes=facet_nodes, outward_normals=normals, sorted_outward_normals=son)
    ev = lambda name, ids: C.FUNCS[name](np, X[ids, 0], X[ids, 1])
    betas = {f: ev(v[1], facet_nodes[f]) for f, v in case["bc"].items() if isinstance(v, tuple)}
    bcv = {f: ev(v[0] if isinstance(v, tuple) else v, facet_nodes[f]) for f, v in case["bc"].items()}
    W = np.zeros((Ni, 5))
    W[:, 3] = W[:, 4] = 1.0
    rows = O.boundary_rows(cl, O.robin_betas(cl, betas))
    K = O.assemble_K(cl, "polyharmonic", 1.0, case["max_degree"], W, rows)
    A = O.assemble_A(cl, "polyharmonic", 1.0, case["max_degree"])
    q = O.assemble_q(cl, C.FUNCS[case["rhs"]](np, X[:Ni, 0], X[:Ni, 1]), bcv)
    u, c, _ = O.solve_faithful(K, A, q)
    assert np.linalg.norm(u - g["vals"]) <= 1e-9 * np.linalg.norm(g["vals"])


def test_gmsh_cloud_rejects_periodic_facets():
    with pytest.raises(NotImplementedError):
        GmshCloud(os.path.join(HERE, "dshape.msh"), facet_types={"Bottom": "p", "Right": "n", "Top": "p", "Left": "d"})
