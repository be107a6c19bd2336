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


def _loss(precision, control=None, fields=None, want_grad=True, case_name=None):
    """J = mean_interior (vals - u_t)^2 + 1e-4 ||control||^2 on the boundary-control golden case (or on its
    local-support version)."""
    import torch

    import updes_gb300 as U
    from updes_gb300.adjoint import pde_solver_torch
    case = C.CASES[C.ADJOINT_CASE] if case_name is None else C.LOCAL_CASES[case_name]
    cl = product_cloud(case)
    g = load("adjoint_kgrad_10x10" if case_name is None else f"adjoint_{case_name}")
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


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_local_support_adjoint_matches_reference_autodiff(precision):
    """The same gradients with local supports (support_size 22): Phi is then sparse and not symmetric, so the
    adjoint's [Phi P]^T g and its operator-weight gradient take the support lists (golden vectors from
    reverse mode through the reference's solve on its BallTree supports)."""
    g = load(f"adjoint_{C.LOCAL_ADJOINT_CASE}")
    J, dc, dF = _loss(precision, case_name=C.LOCAL_ADJOINT_CASE)
    assert abs(J - float(g["J"])) <= 1e-9 * abs(float(g["J"]))
    assert rel(dc, g["dJ_dc"]) < 1e-6
    assert rel(dF, g["dJ_dfields"]) < 1e-6


def test_adjoint_matches_central_differences():
    """Directional derivatives along random directions against central differences.

    The boundary-control workload solves in FP64, so the quotients are taken on the FP64 path.  J is
    exactly quadratic in the control, so h = 1e-2 is exact up to rounding and pins the adjoint at 1e-8.
    At h = 1e-6 the quotient carries the forward solves' rounding divided by 2h: along the control the
    factors are reused and that noise is a few 1e-5 of the derivative (SciPy's LU of the same K gives 3.2e-5
    at h = 1e-6; bound 1e-4); along the fields K itself changes and is refactored, whose rounding (about
    1e-11 of J on this r^5 system) gives about 1e-4 of the derivative (bound 1e-3).  At h = 1e-4 the
    fields' quotient is as close as FP64 difference quotients get on this system (truncation and rounding
    balance near 1e-6: SciPy's LU of the same problem gives 9.5e-7 at h = 1e-4 and 2.3e-6 at 1e-3; bound
    3e-6).  The FP32 path's adjoint is checked along the
    control at h = 1e-2: each of its solves stops at a backward error of 256 FP64 unit roundoffs, so two
    perturbed solves differ by about 1e-10 of J and the quotient by about 1e-8 of the derivative (bound
    1e-7).
    """
    g = load("adjoint_kgrad_10x10")
    case = C.CASES[C.ADJOINT_CASE]
    cl = product_cloud(case)
    F0 = C.make_fields(case, cl.sorted_nodes)
    c0 = g["control"]
    rng = np.random.default_rng(0)
    v = rng.standard_normal(c0.shape)
    V = rng.standard_normal(F0.shape)

    def fd_c(prec, h):
        return (_loss(prec, control=c0 + h * v, want_grad=False) -
                _loss(prec, control=c0 - h * v, want_grad=False)) / (2 * h)

    def fd_f(prec, h):
        return (_loss(prec, fields=F0 + h * V, want_grad=False) -
                _loss(prec, fields=F0 - h * V, want_grad=False)) / (2 * h)

    J, dc, dF = _loss("fp64")
    gc, gf = dc @ v, np.sum(dF * V)
    assert abs(fd_c("fp64", 1e-2) - gc) <= 1e-8 * abs(gc)
    assert abs(fd_c("fp64", 1e-6) - gc) <= 1e-4 * abs(gc)
    assert abs(fd_f("fp64", 1e-4) - gf) <= 3e-6 * abs(gf)
    assert abs(fd_f("fp64", 1e-6) - gf) <= 1e-3 * abs(gf)
    J32, dc32, _ = _loss("fp32")
    assert abs(fd_c("fp32", 1e-2) - dc32 @ v) <= 1e-7 * abs(dc32 @ v)
