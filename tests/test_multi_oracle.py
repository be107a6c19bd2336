"""CPU: the oracle's restatement of pde_multi_solver's Picard sweeps (updes/operators.py:686-771) against
the reference's own outputs on two coupled two-field systems (golden vectors made by running the reference)."""
import os

import numpy as np
import pytest

import cases as C
from oracle import updes_np as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def oracle_multi(case):
    """Every sweep solves both fields' PDEs with the previous sweep's values of both fields as the
    operators' fields (per node) and the old-time values, as coefficients, in the right-hand sides; the
    reference's order of operations (inv -> GEMM -> QR -> inv) for each solve."""
    cloud = O.square_cloud(case["Nx"], case["Ny"], case["facets"], coords=C.grid_coords(case))
    kind, a = "polyharmonic", float(case["rbf"][1])
    deg = case["max_degree"]
    X = cloud.sorted_nodes
    Ni = cloud.Ni
    u0, v0 = C.multi_initial(case, X)
    A = O.assemble_A(cloud, kind, a, deg)
    rows = O.boundary_rows(cloud, {})
    cu, cv = (O.field_coefficients(cloud, kind, a, deg, f) for f in (u0, v0))  # rhs_args -> coefficients
    xi = X[:Ni]
    zero_bc = {f: 0.0 for f in case["facets"]}
    if case["kind"] == "grayscott":
        U, V = O.value(xi, cu, X, kind, a), O.value(xi, cv, X, kind, a)
        rhs = [C.GS_DU * O.laplacian(xi, cu, X, kind, a) - U * V ** 2 + C.GS_F * (1 - U),
               C.GS_DV * O.laplacian(xi, cv, X, kind, a) + U * V ** 2 - (C.GS_F + C.GS_K) * V]
    else:
        rhs = [O.value(xi, cu, X, kind, a) / C.BURGERS_DT, O.value(xi, cv, X, kind, a) / C.BURGERS_DT]
    it = [u0, v0]
    sols = None
    for _ in range(case["nb_iters"]):
        if case["kind"] == "grayscott":
            W = np.zeros((Ni, 5))
            W[:, 0] = 1.0
        else:
            W = np.stack([np.full(Ni, 1.0 / C.BURGERS_DT), it[0][:Ni], it[1][:Ni], np.zeros(Ni), np.zeros(Ni)], 1)
        K = O.assemble_K(cloud, kind, a, deg, W, rows)
        sols = [O.solve_faithful(K, A, O.assemble_q(cloud, rhs[i], zero_bc))[:2] for i in range(2)]
        it = [s[0] for s in sols]
    return sols


@pytest.mark.parametrize("name", list(C.MULTI_CASES))
def test_oracle_multi_solver_matches_reference(name):
    g = np.load(os.path.join(HERE, f"{name}.npz"))
    case = C.MULTI_CASES[name]
    sols = oracle_multi(case)
    for i in range(2):
        u, c = sols[i]
        assert np.linalg.norm(u - g["vals"][i]) <= 1e-9 * np.linalg.norm(g["vals"][i])
        assert np.linalg.norm(c - g["coeffs"][i]) <= 1e-8 * np.linalg.norm(g["coeffs"][i])
