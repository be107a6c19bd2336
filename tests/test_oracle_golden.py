"""The oracle against golden vectors produced by the reference's own code (CPU only)."""
import json

import numpy as np
import pytest

import cases as C
from golden_problem import case_of, load, oracle_problem
from oracle import updes_np as O

NAMES = list(C.CASES) + list(C.LOCAL_CASES)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_cloud_ordering(name):
    g = load(name)
    case = case_of(g)
    p = oracle_problem(case)
    cl = p["cloud"]
    assert np.array_equal(cl.sorted_nodes, g["sorted_nodes"])
    assert [cl.N, cl.Ni, cl.Nd, cl.Nn, cl.Nr, sum(cl.Np)] == g["counts"].tolist()
    assert {f: list(map(int, v)) for f, v in cl.facet_nodes.items()} == json.loads(str(g["facet_nodes"]))
    assert np.array_equal(cl.sorted_outward_normals.reshape(-1, 2), g["sorted_outward_normals"].reshape(-1, 2))
    assert {int(k): v for k, v in json.loads(str(g["robin"])).items()} == pytest.approx(p["robin"])


@pytest.mark.parametrize("name", NAMES)
def test_assembly_entries(name):
    """Assembled entries agree with the reference within 1e-12 (relative to the row scale)."""
    g = load(name)
    p = oracle_problem(case_of(g))
    K = O.assemble_K(p["cloud"], p["kind"], p["param"], p["deg"], p["W"], p["rows"],
                     supports=p["supports"])
    A = O.assemble_A(p["cloud"], p["kind"], p["param"], p["deg"], supports=p["supports"])
    N = p["cloud"].N
    D = K[:N]
    if "diffMat" in g:
        ref_D, ref_A, rows, arows = g["diffMat"], g["A"], np.arange(N), np.arange(A.shape[0])
    else:
        rows = arows = g["diffMat_rows"]
        ref_D, ref_A = g["diffMat_sub"], g["A_sub"]
    scale = np.abs(ref_D).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(D[rows] - ref_D) / scale) < 1e-12
    scale = np.abs(ref_A).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(A[arows] - ref_A) / scale) < 1e-12
    # checksums over every row
    assert np.allclose(D.sum(1), g["diffMat_rowsum"], rtol=1e-11, atol=1e-11 * np.abs(D).sum(1).max())
    assert np.allclose(np.abs(D).sum(1), g["diffMat_rowabs"], rtol=1e-12)
    assert np.allclose(np.abs(A).sum(1), g["A_rowabs"], rtol=1e-12)
    # the Pᵀ block of K equals A's
    assert np.array_equal(K[N:, :N], A[N:, :N])


@pytest.mark.parametrize("name", NAMES)
def test_rhs(name):
    g = load(name)
    p = oracle_problem(case_of(g))
    assert rel(p["q"], g["q"]) < 1e-12


@pytest.mark.parametrize("name", NAMES)
def test_solution_faithful(name):
    """The oracle's restatement of the reference's solve order reproduces vals and coeffs."""
    g = load(name)
    p = oracle_problem(case_of(g))
    K = O.assemble_K(p["cloud"], p["kind"], p["param"], p["deg"], p["W"], p["rows"],
                     supports=p["supports"])
    A = O.assemble_A(p["cloud"], p["kind"], p["param"], p["deg"], supports=p["supports"])
    u, c, B = O.solve_faithful(K, A, p["q"])
    assert rel(u, g["vals"]) < 1e-9
    if "B" in g:
        assert rel(B, g["B"]) < 1e-9


@pytest.mark.parametrize("name", NAMES)
def test_solution_direct(name):
    """One LU of the Kansa matrix gives the reference's solution (formulation check)."""
    g = load(name)
    p = oracle_problem(case_of(g))
    K = O.assemble_K(p["cloud"], p["kind"], p["param"], p["deg"], p["W"], p["rows"],
                     supports=p["supports"])
    A = O.assemble_A(p["cloud"], p["kind"], p["param"], p["deg"], supports=p["supports"])
    u, c = O.solve_direct(K, A, p["q"])
    assert rel(u, g["vals"]) < 1e-8


@pytest.mark.parametrize("name", NAMES)
def test_field_operators(name):
    g = load(name)
    p = oracle_problem(case_of(g))
    X = p["cloud"].sorted_nodes
    v = O.value(X, g["coeffs"], X, p["kind"], p["param"])
    gr = O.gradient(X, g["coeffs"], X, p["kind"], p["param"])
    assert rel(v, g["value_at_nodes"]) < 1e-12
    assert rel(gr, g["grad_at_nodes"]) < 1e-12


@pytest.mark.parametrize("name", list(C.LOCAL_CASES))
def test_local_supports_match_the_reference(name):
    """The k - 1 nearest other nodes of every node, as sets, equal the reference's BallTree supports."""
    g = load(name)
    p = oracle_problem(case_of(g))
    ref = g["sorted_local_supports"]
    assert p["supports"].shape == ref.shape
    assert all(set(a) == set(b) for a, b in zip(p["supports"].tolist(), ref.tolist()))
