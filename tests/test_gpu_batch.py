"""GPU parity of the batched right-hand-side path (updes_solve_batch, updes_eval_values_batch) and of
implicit time stepping under a CUDA graph, against the oracle's FP64 direct solves."""
import ctypes

import numpy as np
import pytest

import cases as C
from golden_problem import oracle_problem
from gpu_helpers import rbf_callable
from oracle import updes_np as O
from test_host import _bcs, _diff_operator, product_cloud
import updes_gb300 as U
from updes_gb300 import _lib
from updes_gb300.multirhs import MultiRHSSolver

pytestmark = pytest.mark.gpu

# FP64 factors: every golden case; FP32 factors: the cases conditioned well enough for six classical sweeps
FP32_CASES = ["readme_laplace_30x20", "poisson_jitter_11x11", "kgrad_fields_10x10", "advdiff_rhsargs_9x9",
              "darcy_mq_8x8", "thinplate_deg4_8x8"]
BATCH_RUNS = [(name, "fp64", 1) for name in C.CASES] + [(name, "fp32", 6) for name in FP32_CASES]


def _solver(case, sweeps, precision="fp64"):
    cl = product_cloud(case)
    fields = C.make_fields(case, cl.sorted_nodes)
    s = MultiRHSSolver(_diff_operator(case["op"]), cl, _bcs(case, cl), rbf_callable(case), case["max_degree"],
                       diff_args=None if fields is None else list(fields), sweeps=sweeps,
                       options=U.SolverOptions(precision=precision))
    return cl, s


def _oracle_solve(case, Q):
    p = oracle_problem(case)
    K = O.assemble_K(p["cloud"], p["kind"], p["param"], p["deg"], p["W"], p["rows"])
    A = O.assemble_A(p["cloud"], p["kind"], p["param"], p["deg"])[:p["cloud"].N]
    n, N = K.shape[0], Q.shape[0]
    B = np.vstack([Q, np.zeros((n - N, Q.shape[1]))])
    Cref = np.linalg.solve(K, B)
    return Cref, A @ Cref, K, B


def _colrel(a, b):
    return (np.linalg.norm(a - b, axis=0) / np.maximum(np.linalg.norm(b, axis=0), 1e-300)).max()


def _backward_error(K, C, B):
    """max over columns of ||K c - b|| / (||K|| ||c|| + ||b||) (normwise, 2-norms)."""
    nK = np.linalg.norm(K, 2)
    r = K @ C - B
    return (np.linalg.norm(r, axis=0) / (nK * np.linalg.norm(C, axis=0) + np.linalg.norm(B, axis=0))).max()


@pytest.mark.parametrize("name,precision,sweeps", BATCH_RUNS)
@pytest.mark.parametrize("R", [1, 7, 64])
def test_batch_solve_matches_oracle(name, precision, sweeps, R):
    """R random right-hand sides: vals within 1e-8 of the oracle's FP64 direct solves, on FP64 factors as
    double-float planes (one sweep) and on FP32 factors (six sweeps), and coefficients with a normwise
    backward error below 1e-13 (the coefficients themselves are as ill-determined as K).  The residual is
    double-float (about 2^-48 of |K||c|), so refinement settles within kappa * 2^-48 of the solution."""
    case = C.CASES[name]
    cl, s = _solver(case, sweeps=sweeps, precision=precision)
    Q = np.random.default_rng(R).standard_normal((cl.N, R))
    Cg, Vg = s.solve(Q)
    Cref, Vref, K, B = _oracle_solve(case, Q)
    assert _colrel(Vg.cpu().numpy(), Vref) < 1e-8
    assert _backward_error(K, Cg.cpu().numpy(), B) < 1e-13


def test_batch_agrees_with_single_rhs_path():
    """Each column's vals equal the single right-hand-side FP64 solve to 1e-8."""
    case = C.CASES["readme_laplace_30x20"]
    cl, s = _solver(case, sweeps=1)
    Q = np.random.default_rng(5).standard_normal((cl.N, 3))
    _, Vg = s.solve(Q)
    for j in range(3):
        _, v1, _ = U.operators.solve_device(s.dp, Q[:, j], s.opts, want_vals=True)
        a, b = Vg[:, j].cpu().numpy(), v1.cpu().numpy()
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b)


def test_batch_sweeps_reduce_error():
    """On FP32 factors each sweep of classical refinement shrinks the backward error until it reaches
    the FP64 level."""
    case = C.CASES["poisson_jitter_11x11"]
    cl, s = _solver(case, sweeps=0, precision="fp32")
    Q = np.random.default_rng(1).standard_normal((cl.N, 4))
    _, _, K, B = _oracle_solve(case, Q)
    errs = []
    for sw in (0, 1, 2, 4):
        s.sweeps = sw
        errs.append(_backward_error(K, s.solve(Q, want_vals=False)[0].cpu().numpy(), B))
    assert errs[0] > 1e-12 and errs[1] < errs[0] / 10
    assert errs[-1] < 1e-13


def test_eval_values_batch_matches_single():
    import torch
    case = C.CASES["gaussian_dnr_9x8"]
    cl, s = _solver(case, sweeps=2)
    lib = _lib.load()
    R = 33
    Cm = torch.as_tensor(np.random.default_rng(3).standard_normal((s.n, R)), device="cuda")
    V = torch.empty((s.N, R), dtype=torch.float64, device="cuda")
    _lib.check(lib.updes_eval_values_batch(ctypes.byref(s.dp.c), R, Cm.data_ptr(), R, V.data_ptr(), R,
                                           s.dp.stream()), "updes_eval_values_batch")
    for j in (0, 17, 32):
        c = Cm[:, j].contiguous()
        v = torch.empty(s.N, dtype=torch.float64, device="cuda")
        _lib.check(lib.updes_eval_values(ctypes.byref(s.dp.c), c.data_ptr(), v.data_ptr(), s.dp.stream()),
                   "updes_eval_values")
        a, b = V[:, j].cpu().numpy(), v.cpu().numpy()
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


def test_batch_rejects_unfactored_workspace():
    """A workspace without factors of this system: the device check reports UPDES_ERR_INVALID."""
    import torch
    case = C.CASES["readme_laplace_30x20"]
    cl, s = _solver(case, sweeps=1)
    s.ws.zero_()  # wipe the factor state (a host-side mistake, caught on the device)
    with pytest.raises(_lib.UpdesError):
        s.solve(np.ones((cl.N, 2)))
    torch.cuda.synchronize()


def test_batch_invalid_arguments():
    case = C.CASES["readme_laplace_30x20"]
    cl, s = _solver(case, sweeps=1)
    with pytest.raises(ValueError):
        s.solve(np.ones((cl.N, 65)))
    lib = _lib.load()
    st = lib.updes_solve_batch(ctypes.byref(s.dp.c), 0, None, 1, None, 1, 1, s.ws.data_ptr(), s.ws.numel(),
                               s.bws.data_ptr(), s.bws.numel(), s.dp.stream())
    assert st == _lib.ERR_INVALID
    st = lib.updes_solve_batch(ctypes.byref(s.dp.c), 2, s.ws.data_ptr(), 2, s.ws.data_ptr(), 2, 1, s.ws.data_ptr(),
                               s.ws.numel(), s.bws.data_ptr(), 16, s.dp.stream())
    assert st == _lib.ERR_WORKSPACE


def _advection_case(Nx):
    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    cl = U.SquareCloud(Nx=Nx, Ny=Nx, facet_types=facets)
    dt, kappa, vel = 1e-3, 0.01, (1.0, 0.5)

    def op(x, center, rbf, monomial, fields=None):
        v = U.nodal_value(x, center, rbf, monomial)
        g = U.nodal_gradient(x, center, rbf, monomial)
        lap = U.nodal_laplacian(x, center, rbf, monomial)
        return v / dt + vel[0] * g[0] + vel[1] * g[1] - kappa * lap
    bcs = {f: np.zeros(len(cl.facet_nodes[f])) for f in facets}
    return cl, op, bcs, dt


def test_implicit_steps_graph_equals_eager_and_oracle():
    """Three implicit-Euler steps of advection-diffusion for 5 bumps: the graph replay equals the eager
    launches bit for bit, and both follow the oracle's FP64 steps to 1e-8."""
    cl, op, bcs, dt = _advection_case(16)
    rbf = U.polyharmonic
    s = MultiRHSSolver(op, cl, bcs, rbf, 1, sweeps=1)
    X = cl.sorted_nodes
    rng = np.random.default_rng(0)
    cen = rng.uniform(0.3, 0.7, (5, 2))
    wid = rng.uniform(0.05, 0.15, 5)
    U0 = np.exp(-((X[:, None, 0] - cen[None, :, 0]) ** 2 + (X[:, None, 1] - cen[None, :, 1]) ** 2)
                / (2 * wid[None, :] ** 2))
    Ug = s.implicit_steps(U0, 3, 1.0 / dt, graph=True).cpu().numpy()
    Ue = s.implicit_steps(U0, 3, 1.0 / dt, graph=False).cpu().numpy()
    assert np.array_equal(Ug, Ue)
    # oracle
    Ni = cl.Ni
    W = np.zeros((Ni, 5))
    W[:, 0], W[:, 1], W[:, 2], W[:, 3], W[:, 4] = 1 / dt, 1.0, 0.5, -0.01, -0.01
    ocl = O.square_cloud(16, 16, {"South": "d", "West": "d", "North": "d", "East": "d"})
    assert np.array_equal(ocl.sorted_nodes, X)
    K = O.assemble_K(ocl, "polyharmonic", 1, 1, W, O.boundary_rows(ocl, {}))
    A = O.assemble_A(ocl, "polyharmonic", 1, 1)[:cl.N]
    Uo = U0.copy()
    for _ in range(3):
        Q = np.zeros_like(Uo)
        Q[:Ni] = Uo[:Ni] / dt
        Cs = np.linalg.solve(K, np.vstack([Q, np.zeros((K.shape[0] - cl.N, Q.shape[1]))]))
        Uo = A @ Cs
    assert _colrel(Ug, Uo) < 1e-8
