"""Parity at the benchmark configurations' own sizes, against the FP64 oracle run on the CPU.

The fixtures come from ``tests/golden/make_fullsize.py`` (the oracle of ``oracle/updes_np.py``, itself
pinned to the reference's outputs on the small golden cases):

* N = 22,500 Poisson (the headline workload): vals of the mixed path within 1e-8 and of the FP64 path within
  1e-10 of the oracle's direct LU, both within 1e-8 (or 3x the measured distance between the two CPU solve
  orders, whichever is larger) of the reference's own operation order (inv -> GEMM -> QR) run by the
  oracle; coefficients through their backward error on the assembled K and their distance to the oracle's.
* N = 10,000 boundary control (r^5, FP64): J, dJ/dc and dJ/d(fields) against a dense FP64 adjoint, and the
  adjoint's directional derivatives against central differences of the GPU solve.
* N = 6,400 advection-diffusion: the first implicit step of all 64 bumps against the oracle.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _fixture(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip(f"{name} not generated (tests/golden/make_fullsize.py)")
    return dict(np.load(path))


@pytest.fixture(scope="module")
def poisson_problem():
    import torch

    import updes_gb300 as U
    from updes_gb300 import workloads as WL
    sysd = WL.poisson_manufactured(150)
    opts = U.SolverOptions(precision="fp32", reuse_factorization=False)
    W, kind, bnodes, geom, q = U.operators.prepare(sysd["diff_operator"], sysd["rhs_operator"], sysd["cloud"],
                                                   sysd["boundary_conditions"], sysd["rbf"], 2, options=opts)
    dp = U.operators.DeviceProblem(sysd["cloud"], sysd["rbf"], 2, W, kind, bnodes, geom)
    yield sysd, dp, torch.as_tensor(q, device="cuda")
    U.operators.free_workspace()
    torch.cuda.empty_cache()


def _backward_error(dp, coeffs, q):
    """max_i |K c - b|_i / max_i (|K| |c| + |b|)_i on the FP64 K assembled by the library."""
    import torch

    from updes_gb300 import _lib
    lib = _lib.load()
    ld = int(lib.updes_matrix_ld(dp.n, 8))
    K = torch.zeros((dp.n, ld), dtype=torch.float64, device="cuda")
    _lib.check(lib.updes_assemble(ctypes.byref(dp.c), K.data_ptr(), ld, None, 0, dp.stream()), "updes_assemble")
    Kv = K[:, :dp.n]
    b = torch.cat([q, torch.zeros(dp.n - dp.N, dtype=torch.float64, device="cuda")])
    out = []
    for c in coeffs:
        c = torch.as_tensor(c, dtype=torch.float64, device="cuda")
        r = (Kv @ c - b).abs()
        scale = Kv.abs() @ c.abs() + b.abs()
        out.append(float(r.max() / scale.max()))
    del K, Kv
    torch.cuda.empty_cache()
    return out


def test_headline_poisson_against_oracle(poisson_problem):
    import updes_gb300 as U
    g = _fixture("full_poisson_150.npz")
    sysd, dp, qd = poisson_problem
    X = sysd["cloud"].sorted_nodes
    np.testing.assert_allclose(g["sorted_nodes_digest"], [X.sum(), (X * X).sum()], rtol=1e-14)
    res = {}
    for prec in ("fp32", "fp64"):
        c, v, info = U.operators.solve_device(dp, qd, U.SolverOptions(precision=prec, reuse_factorization=False))
        res[prec] = (c.cpu().numpy(), v.cpu().numpy(), info)
    e32, e64 = rel(res["fp32"][1], g["vals"]), rel(res["fp64"][1], g["vals"])
    print(f"vals vs oracle direct LU: mixed {e32:.3e}, FP64 {e64:.3e}; GMRES iterations {res['fp32'][2]['iters']}")
    assert res["fp32"][2]["fell_back"] == 0
    assert e32 <= 1e-8
    assert e64 <= 1e-10
    if "vals_faithful" in g:
        floor = rel(g["vals_faithful"], g["vals"])
        for prec in ("fp32", "fp64"):
            ef = rel(res[prec][1], g["vals_faithful"])
            print(f"{prec} vals vs the reference's order of operations: {ef:.3e} (CPU floor {floor:.3e})")
            assert ef <= max(1e-8, 3 * floor)
    # coefficients: backward error of each on the same K; distance to the oracle's coefficients
    be = _backward_error(dp, [res["fp32"][0], res["fp64"][0], g["coeffs"]], qd)
    print(f"coeffs backward error: mixed {be[0]:.2e}, FP64 {be[1]:.2e}, oracle {be[2]:.2e}; "
          f"rel diff to oracle: mixed {rel(res['fp32'][0], g['coeffs']):.2e}, "
          f"FP64 {rel(res['fp64'][0], g['coeffs']):.2e}")
    assert be[0] <= 1e-13 and be[1] <= 1e-13
    assert be[0] <= 100 * max(be[2], 1e-16) and be[1] <= 100 * max(be[2], 1e-16)


def _control_loss(sysd, F, ctl_np, want_grad=True, precision="fp64"):
    import torch

    import updes_gb300 as U
    from updes_gb300.adjoint import pde_solver_torch
    cl = sysd["cloud"]
    ctl = torch.tensor(ctl_np, device="cuda", requires_grad=want_grad)
    ft = [torch.tensor(f, device="cuda", requires_grad=want_grad) for f in F]
    bcs = dict(sysd["boundary_conditions"])
    bcs["North"] = ctl
    vals, _ = pde_solver_torch(sysd["diff_operator"], sysd["rhs_operator"], cl, bcs, sysd["rbf"],
                               sysd["max_degree"], diff_args=ft, options=U.SolverOptions(precision=precision))
    X = cl.sorted_nodes
    ut = torch.tensor(np.sinh(np.pi * X[:, 1]) * np.sin(np.pi * X[:, 0]) / np.sinh(np.pi), device="cuda")
    Ni = cl.Ni
    J = torch.mean((vals[:Ni] - ut[:Ni]) ** 2) + 1e-4 * torch.sum(ctl ** 2)
    if not want_grad:
        return float(J)
    J.backward()
    return float(J), ctl.grad.cpu().numpy(), np.stack([f.grad.cpu().numpy() for f in ft]), vals.detach().cpu().numpy()


def test_boundary_control_adjoint_against_oracle():
    """N = 10,000, r^5, FP64, the first seeded control.  The dense FP64 oracle and the GPU agree on J to
    1e-10 and on both gradients to 1e-6; the adjoint's directional derivatives match central differences
    of the GPU solve to 1e-6: along the control J is exactly quadratic (h = 1e-2, no truncation, the
    factors' rounding cancels between the two solves), along the fields a Richardson combination of
    h = 1e-3 and 5e-4 removes the O(h^2) term."""
    from updes_gb300 import workloads as WL
    g = _fixture("full_control_100.npz")
    sysd, F, controls, _ = WL.boundary_control(100, 32)
    np.testing.assert_array_equal(controls[0], g["control"])
    J, dc, dF, vals = _control_loss(sysd, F, controls[0])
    ej, ec, ef = abs(J - float(g["J"])) / abs(float(g["J"])), rel(dc, g["dJ_dc"]), rel(dF, g["dJ_dfields"])
    print(f"control N=10,000: J rel {ej:.2e}, dJ/dc rel {ec:.2e}, dJ/dfields rel {ef:.2e}, "
          f"vals rel {rel(vals, g['vals']):.2e}")
    assert ej <= 1e-10
    assert ec <= 1e-6
    assert ef <= 1e-6
    rng = np.random.default_rng(5)
    v = rng.standard_normal(controls[0].shape)
    V = rng.standard_normal(np.shape(F))
    h = 1e-2
    fd_c = (_control_loss(sysd, F, controls[0] + h * v, False) - _control_loss(sysd, F, controls[0] - h * v, False)) \
        / (2 * h)
    gc = float(dc @ v)

    def fd_f(hh):
        Fp = [f + hh * d for f, d in zip(F, V)]
        Fm = [f - hh * d for f, d in zip(F, V)]
        return (_control_loss(sysd, Fp, controls[0], False) - _control_loss(sysd, Fm, controls[0], False)) / (2 * hh)
    f1, f2 = fd_f(1e-3), fd_f(5e-4)
    fd_fr = (4 * f2 - f1) / 3
    gf = float(np.sum(dF * V))
    print(f"central differences: control {abs(fd_c - gc) / abs(gc):.2e}, fields "
          f"{abs(fd_fr - gf) / abs(gf):.2e} (h = 1e-3 alone {abs(f1 - gf) / abs(gf):.2e})")
    assert abs(fd_c - gc) <= 1e-6 * abs(gc)
    assert abs(fd_fr - gf) <= 1e-6 * abs(gf)


def test_advection_first_step_against_oracle():
    """N = 6,400 advection-diffusion, all 64 bumps, one implicit step through the batched solve (FP64
    factors, one refinement sweep) against the oracle's direct LU: 8 columns in full, every column's norm
    and its dot product with a seeded random vector, each within 1e-8."""
    import torch

    from updes_gb300 import workloads as WL
    from updes_gb300.multirhs import MultiRHSSolver
    g = _fixture("full_advection_80.npz")
    sysd, U0, dt = WL.advection_bumps(80, 64)
    solver = MultiRHSSolver(sysd["diff_operator"], sysd["cloud"], sysd["boundary_conditions"], sysd["rbf"],
                            sysd["max_degree"], sweeps=1)
    U1 = solver.implicit_steps(torch.as_tensor(U0, device="cuda"), 1, 1.0 / dt, graph=False).cpu().numpy()
    e_cols = rel(U1[:, :8], g["U1_cols"])
    e_norm = float(np.max(np.abs(np.linalg.norm(U1, axis=0) - g["col_norms"]) / g["col_norms"]))
    dots = g["probe"] @ U1
    e_dot = float(np.max(np.abs(dots - g["col_dots"]) / (np.linalg.norm(g["probe"]) * g["col_norms"])))
    print(f"advection step 1: 8 columns {e_cols:.2e}, norms {e_norm:.2e}, probes {e_dot:.2e}")
    assert e_cols <= 1e-8 and e_norm <= 1e-8 and e_dot <= 1e-8
