"""GPU: the reference's assembly functions by name (updes_gb300.assembly) against the reference's own
matrices on every golden case: [opΦ opP; bdΦ bdP] (diffMat), A, q at 1e-12 of each row's largest entry; B and
inv(A) through their defining products."""
import json

import numpy as np
import pytest

import cases as C
from golden_problem import case_of, load
from gpu_helpers import rbf_callable, rhs_operator
from test_host import _bcs, _diff_operator, product_cloud
from updes_gb300 import assembly as AS

pytestmark = pytest.mark.gpu
NAMES = list(C.CASES)


def _rowrel(got, ref):
    scale = np.abs(ref).max(axis=1, keepdims=True) + 1e-300
    return float(np.max(np.abs(got - ref) / scale))


@pytest.mark.parametrize("name", NAMES)
def test_assembly_functions_match_the_reference(name):
    g = load(name)
    case = case_of(g)
    cl = product_cloud(case)
    rbf = rbf_callable(case)
    M = {0: 1, 1: 3, 2: 6, 3: 10, 4: 15}[case["max_degree"]]
    fields = C.make_fields(case, cl.sorted_nodes)
    args = None if fields is None else list(fields)
    robin = {int(k): float(v) for k, v in json.loads(str(g["robin"])).items()}
    opPhi, opP = AS.assemble_op_Phi_P(_diff_operator(case["op"]), cl, rbf, M, args)
    bdPhi, bdP = AS.assemble_bd_Phi_P(cl, rbf, M, robin)
    diff = np.vstack([np.hstack([opPhi, opP]), np.hstack([bdPhi, bdP])])
    if "diffMat" in g:
        ref, rows = g["diffMat"], np.arange(cl.N)
    else:
        ref, rows = g["diffMat_sub"], g["diffMat_rows"]
    assert _rowrel(diff[rows], ref) < 1e-12
    A = AS.assemble_A(cl, rbf, M)
    if "A" in g:
        assert _rowrel(A, g["A"]) < 1e-12
    assert np.array_equal(AS.assemble_Phi(cl, rbf), A[:cl.N, :cl.N])
    assert np.array_equal(AS.assemble_P(cl, M), A[:cl.N, cl.N:])
    rf = C.make_rhs_field(case, cl.sorted_nodes)
    q = AS.assemble_q(rhs_operator(case), _bcs(case, cl), cl, rbf, M, None if rf is None else [rf])
    assert np.linalg.norm(q - g["q"]) <= 1e-12 * np.linalg.norm(g["q"])


def test_inverse_and_B_through_their_definitions():
    g = load("poisson_jitter_11x11")
    case = case_of(g)
    cl = product_cloud(case)
    rbf = rbf_callable(case)
    M = {0: 1, 1: 3, 2: 6, 3: 10, 4: 15}[case["max_degree"]]
    A = AS.assemble_A(cl, rbf, M)
    Ainv = AS.assemble_invert_A(cl, rbf, M)
    resid = np.abs(A @ Ainv - np.eye(A.shape[0])).max()
    assert resid < 1e-9 * np.linalg.cond(A) ** 0.5, resid
    robin = {int(k): float(v) for k, v in json.loads(str(g["robin"])).items()}
    fields = C.make_fields(case, cl.sorted_nodes)
    B = AS.assemble_B(_diff_operator(case["op"]), cl, rbf, M, None if fields is None else list(fields), robin)
    assert np.linalg.norm(B - g["B"]) <= 1e-9 * np.linalg.norm(g["B"])

