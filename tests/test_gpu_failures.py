"""Failure handling on the GPU, made on the host: no test here faults, traps or hangs a GPU.

* A bounded wait that runs out: the polls allowed to the waits between CTAs are cut to one
  (``updes_set_spin_limit``), so the blocks of a multi-block triangular solve give up waiting for their
  predecessors; the call must come back with UPDES_ERR_TIMEOUT, and with the default limit restored the
  same solve on the same context must succeed.
* The FP32 -> FP64 fallback: a refinement capped at one iteration cannot reach the stopping test, so the
  solve refactors in FP64; the result must then be FP64-accurate.
* Bad problems from the host side: two nodes at the same place (an exactly singular Kansa matrix), NaN in
  an operator's coefficient field, and a Gaussian kernel so flat that its system is numerically singular
  in FP32.  Each must end in an error status or a converged FP64-quality answer, never a crash.
"""
import ctypes

import numpy as np
import pytest

import cases as C
import updes_gb300 as U
from golden_problem import load
from gpu_helpers import lu_factor_random as _factor
from gpu_helpers import solve_case
from updes_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_short_spin_limit_returns_timeout_and_context_stays_usable():
    import torch
    lib = _lib.load()
    n = 4096  # 32 blocks of 128 rows: every block but the first waits for the one before it
    A, F, ld, piv, ws, s = _factor(n, 1, 21)
    b = np.random.default_rng(3).standard_normal(n)
    try:
        _lib.set_spin_limit(1)
        bd = torch.as_tensor(b.copy(), device="cuda")
        st = lib.updes_lu_solve(n, F.data_ptr(), ld, 1, piv.data_ptr(), bd.data_ptr(), 1, 1, 0, ws.data_ptr(),
                                ws.numel(), s)
        torch.cuda.synchronize()
    finally:
        _lib.set_spin_limit(0)
    assert st == _lib.ERR_TIMEOUT, _lib.status_string(st)
    bd = torch.as_tensor(b.copy(), device="cuda")
    st = lib.updes_lu_solve(n, F.data_ptr(), ld, 1, piv.data_ptr(), bd.data_ptr(), 1, 1, 0, ws.data_ptr(),
                            ws.numel(), s)
    assert st == _lib.OK, _lib.status_string(st)
    x = bd.cpu().numpy()
    want = np.linalg.solve(A, b)
    assert np.linalg.norm(x - want) <= 1e-3 * np.linalg.norm(want)  # FP32 factors, no refinement


def test_spin_limit_rejects_negative_values():
    assert _lib.load().updes_set_spin_limit(-1) == _lib.ERR_INVALID


def test_refinement_cap_forces_fp64_fallback():
    """One GMRES iteration cannot take the README system (condition number 2.4e9) from its FP32 factors to the
    stopping test, so the solve refactors in FP64; vals then match the reference's to FP64 quality."""
    g = load("readme_laplace_30x20")
    case = C.CASES["readme_laplace_30x20"]
    _, sol = solve_case(case, "fp32", max_iters=1, reuse_factorization=False)
    info = dict(U.LAST_INFO)
    assert info["fell_back"] == 1 and info["converged"] == 1, info
    assert np.linalg.norm(sol.vals - g["vals"]) <= 1e-9 * np.linalg.norm(g["vals"])


def _duplicate_node_system():
    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    nx = 12
    xs = np.linspace(0, 1, nx)
    ii, jj = np.divmod(np.arange(nx * nx), nx)
    coords = np.stack([xs[ii], xs[jj]], -1)
    a, b = 5 * nx + 5, 5 * nx + 6  # two interior nodes
    coords[b] = coords[a]
    cloud = U.SquareCloud(Nx=nx, Ny=nx, facet_types=facets, coords=coords)
    op = lambda x, center, rbf, monomial, fields: U.nodal_laplacian(x, center, rbf, monomial)
    rhs = lambda x, centers, rbf, fields: 1.0 + 0.0 * x[0]
    return cloud, op, rhs, {f: (lambda c: 0.0 * c[0]) for f in facets}


def test_duplicate_nodes_are_rejected_on_the_host():
    cloud, op, rhs, bcs = _duplicate_node_system()
    with pytest.raises(ValueError, match="coincide"):
        U.pde_solver(op, rhs, cloud, bcs, U.polyharmonic, 1)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_duplicate_nodes_through_the_c_abi(precision):
    """Two interior nodes at the same coordinates give two identical rows of K (condition number ~1e19).
    Handed straight to updes_solve, the elimination meets a pivot at rounding level, not an exact zero (as
    LAPACK's getrf does on the same matrix).  The call must come back with an error status, or with OK and
    a finite backward error in its report (the FP64 path, like getrs, does not judge its answer; that is why
    the host layer rejects such clouds), must not crash, and must leave the context usable."""
    import torch
    cloud, op, rhs, bcs = _duplicate_node_system()
    o = U.SolverOptions(precision=precision, reuse_factorization=False)
    W, kind, bnodes, geom, q = U.operators.prepare(op, rhs, U.SquareCloud(Nx=12, Ny=12, facet_types=dict(
        cloud.facet_types)), bcs, U.polyharmonic, 1, options=o)
    dp = U.operators.DeviceProblem(cloud, U.polyharmonic, 1, W, kind, bnodes, geom)
    try:
        _, _, info = U.operators.solve_device(dp, q, o)
        print(precision, info)
        assert np.isfinite(info["backward_error"]), info
    except _lib.UpdesError as e:
        assert e.status in (_lib.ERR_SINGULAR, _lib.ERR_NOT_CONVERGED), str(e)
    torch.cuda.synchronize()
    sol = solve_case(C.CASES["poisson_jitter_11x11"], precision, reuse_factorization=False)[1]
    g = load("poisson_jitter_11x11")
    assert np.linalg.norm(sol.vals - g["vals"]) <= 1e-8 * np.linalg.norm(g["vals"])


def test_nan_coefficient_field_is_rejected_on_the_host():
    case = C.CASES["kgrad_fields_10x10"]
    cl = U.SquareCloud(Nx=10, Ny=10, facet_types=case["facets"])
    F = C.make_fields(case, cl.sorted_nodes)
    F[0, 7] = np.nan
    op = lambda x, center, rbf, monomial, fields: (fields[0] * U.nodal_laplacian(x, center, rbf, monomial)
                                                   + fields[1] * U.nodal_gradient(x, center, rbf, monomial)[0])
    bcs = {f: (lambda c: 0.0 * c[0]) for f in case["facets"]}
    with pytest.raises(ValueError, match="not finite"):
        U.pde_solver(op, lambda x, centers, rbf, fields: 0.0 * x[0], cl, bcs, U.polyharmonic, 2,
                     diff_args=list(F))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_nan_weights_through_the_c_abi_give_an_error_status(precision):
    """The same NaN handed straight to updes_solve (no host check): the factorisation flags the non-finite
    pivot and the call returns an error status instead of a result."""
    import torch

    from gpu_helpers import device_problem
    cl, dp, q = device_problem(C.CASES["poisson_jitter_11x11"])
    dp.W[3, 3] = float("nan")
    with pytest.raises(_lib.UpdesError) as ei:
        U.operators.solve_device(dp, q, U.SolverOptions(precision=precision, reuse_factorization=False))
    assert ei.value.status in (_lib.ERR_SINGULAR, _lib.ERR_NOT_CONVERGED), str(ei.value)
    torch.cuda.synchronize()


def test_flat_gaussian_falls_back_or_converges():
    """Gaussian kernel with eps = 0.5 on a 16 x 16 cloud: the condition number is far beyond what FP32
    factors can precondition.  The mixed path must fall back to FP64 and then agree with the FP64 path's
    backward error (its vals are as ill-determined as the system, so they are not compared)."""
    facets = {"South": "d", "West": "n", "North": "d", "East": "d"}
    cloud = U.SquareCloud(Nx=16, Ny=16, facet_types=facets, jitter=(0.2, 3))
    op = lambda x, center, rbf, monomial, fields: U.nodal_laplacian(x, center, rbf, monomial)
    rhs = lambda x, centers, rbf, fields: np.sin(3 * x[0]) + 0.0 * x[1]
    bcs = {f: (lambda c: c[0] * c[1]) for f in facets}
    from functools import partial
    rbf = partial(U.gaussian, eps=0.5)
    out = {}
    for prec in ("fp64", "fp32"):
        try:
            U.pde_solver(op, rhs, cloud, bcs, rbf, 1, options=U.SolverOptions(precision=prec,
                                                                             reuse_factorization=False))
            out[prec] = dict(U.LAST_INFO)
        except _lib.UpdesError as e:
            out[prec] = {"status": e.status, **U.LAST_INFO}
    print(out)
    assert out["fp32"].get("fell_back") == 1 or out["fp32"].get("converged") == 1, out
    if "status" not in out["fp32"]:
        assert out["fp32"]["backward_error"] <= max(1e-13, 10 * out["fp64"]["backward_error"])
