"""Adjoint through the GPU solve: against the reference's own reverse-mode gradient and finite differences."""
import numpy as np
import pytest

import cases as C
from golden_problem import load
from gpu_helpers import rbf_callable, rhs_operator
from test_host import _bcs, _diff_operator, product_cloud

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def _loss(precision, control=None, fields=None, want_grad=True):
    """J = mean_interior (vals - u_t)^2 + 1e-4 ||control||^2 on the boundary-control golden case."""
    import torch

    import updes_gb300 as U
    from updes_gb300.adjoint import pde_solver_torch
    case = C.CASES[C.ADJOINT_CASE]
    cl = product_cloud(case)
    g = load("adjoint_kgrad_10x10")
    ctl = torch.tensor(g["control"] if control is None else control, device="cuda", requires_grad=want_grad)
    F = C.make_fields(case, cl.sorted_nodes) if fields is None else fields
    ft = [torch.tensor(f, device="cuda", requires_grad=want_grad) for f in F]
    bcs = _bcs(case, cl)
    bcs["North"] = ctl
    vals, coeffs = pde_solver_torch(_diff_operator(case["op"]), rhs_operator(case), cl, bcs, rbf_callable(case),
                                    case["max_degree"], diff_args=ft, options=U.SolverOptions(precision=precision))
    X = cl.sorted_nodes
    ut = torch.tensor(C.adjoint_target(np, X[:, 0], X[:, 1]), device="cuda")
    Ni = cl.Ni
    J = torch.mean((vals[:Ni] - ut[:Ni]) ** 2) + C.ADJOINT_REG * torch.sum(ctl ** 2)
    if want_grad:
        J.backward()
        return float(J), ctl.grad.cpu().numpy(), np.stack([f.grad.cpu().numpy() for f in ft])
    return float(J)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_adjoint_matches_reference_autodiff(precision):
    """dJ/d(North Dirichlet values) and dJ/d(k, dk/dx, dk/dy) against jax-style reverse mode through the
    reference's own inv -> GEMM -> QR solve (golden vectors made by importing the reference)."""
    g = load("adjoint_kgrad_10x10")
    J, dc, dF = _loss(precision)
    assert abs(J - float(g["J"])) <= 1e-9 * abs(float(g["J"]))
    assert rel(dc, g["dJ_dc"]) < 1e-6
    assert rel(dF, g["dJ_dfields"]) < 1e-6


def test_adjoint_matches_central_differences():
    """Directional derivatives along random directions, central differences with h = 1e-6."""
    g = load("adjoint_kgrad_10x10")
    case = C.CASES[C.ADJOINT_CASE]
    cl = product_cloud(case)
    F0 = C.make_fields(case, cl.sorted_nodes)
    c0 = g["control"]
    J, dc, dF = _loss("fp32")
    rng = np.random.default_rng(0)
    h = 1e-6
    v = rng.standard_normal(c0.shape)
    fd = (_loss("fp32", control=c0 + h * v, want_grad=False) - _loss("fp32", control=c0 - h * v, want_grad=False)) / (2 * h)
    assert abs(fd - dc @ v) <= 1e-6 * abs(dc @ v) + 1e-12
    V = rng.standard_normal(F0.shape)
    fd = (_loss("fp32", fields=F0 + h * V, want_grad=False) - _loss("fp32", fields=F0 - h * V, want_grad=False)) / (2 * h)
    assert abs(fd - np.sum(dF * V)) <= 1e-6 * abs(np.sum(dF * V)) + 1e-12
