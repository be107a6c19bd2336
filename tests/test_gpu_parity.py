"""GPU parity: the CUDA path through the C ABI against the oracle and the reference's golden vectors."""
import ctypes

import numpy as np
import pytest

import cases as C
from golden_problem import case_of, load, oracle_problem
from gpu_helpers import assemble, device_problem, solve_case
from oracle import updes_np as O
from updes_gb300 import _lib

pytestmark = pytest.mark.gpu
NAMES = list(C.CASES) + list(C.LOCAL_CASES)


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("compat", [True, False])
def test_assembly_matches_oracle(name, compat):
    """Every assembled entry within 1e-12 of the oracle, relative to its row's scale."""
    case = case_of(load(name))
    p = oracle_problem(case, compat=compat)
    K = O.assemble_K(p["cloud"], p["kind"], p["param"], p["deg"], p["W"], p["rows"], supports=p["supports"])
    cl, dp, q = device_problem(case, compat=compat)
    K64, K32, ld = assemble(dp, fp32=True)
    Kg = K64.cpu().numpy()
    n = dp.n
    assert np.all(Kg[:, n:] == 0.0)
    Kg = Kg[:, :n]
    scale = np.abs(K).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(Kg - K) / scale) < 1e-12
    assert np.array_equal(K32.cpu().numpy()[:, :n], Kg.astype(np.float32))
    assert np.allclose(q, p["q"], rtol=1e-12, atol=1e-12 * np.abs(p["q"]).max())


@pytest.mark.parametrize("name", NAMES)
def test_assembly_against_reference_rows(name):
    """The same entries against the reference's own matrices (golden)."""
    g = load(name)
    case = case_of(g)
    cl, dp, q = device_problem(case)
    K64, _, _ = assemble(dp)
    Kg = K64.cpu().numpy()[:cl.N, :dp.n]
    if "diffMat" in g:
        ref, rows = g["diffMat"], np.arange(cl.N)
    else:
        ref, rows = g["diffMat_sub"], g["diffMat_rows"]
    scale = np.abs(ref).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(Kg[rows] - ref) / scale) < 1e-12
    assert rel(q, g["q"]) < 1e-12


@pytest.mark.parametrize("name", NAMES)
def test_eval_kernels(name):
    import torch
    g = load(name)
    case = case_of(g)
    cl, dp, q = device_problem(case)
    lib = _lib.load()
    c = torch.as_tensor(g["coeffs"], device="cuda")
    vals = torch.empty(cl.N, dtype=torch.float64, device="cuda")
    _lib.check(lib.updes_eval_values(ctypes.byref(dp.c), c.data_ptr(), vals.data_ptr(), dp.stream()), "eval")
    p = oracle_problem(case)
    want = O.eval_values(p["cloud"], p["kind"], p["param"], p["deg"], g["coeffs"], supports=p["supports"])
    assert rel(vals.cpu().numpy(), want) < 1e-12
    import updes_gb300 as U
    from gpu_helpers import rbf_callable
    X = cl.sorted_nodes
    assert rel(U.value_vec(X, g["coeffs"], X, rbf_callable(case)), g["value_at_nodes"]) < 1e-12
    assert rel(U.gradient_vec(X, g["coeffs"], X, rbf_callable(case)), g["grad_at_nodes"]) < 1e-12
    lap = U.laplacian_vec(X, g["coeffs"], X, rbf_callable(case))
    t = O.rbf_terms(p["kind"], p["param"], X[:, 0:1] - X[None, :, 0], X[:, 1:2] - X[None, :, 1])
    want_lap = (t[3] + t[4]) @ g["coeffs"][:cl.N] + sum(
        g["coeffs"][cl.N + k] * (lambda m: m[3] + m[4])(O.monomial_terms(k, X[:, 0], X[:, 1]))
        for k in range(dp.M))
    assert rel(lap, want_lap) < 1e-12


def _floor(g, p):
    K = O.assemble_K(p["cloud"], p["kind"], p["param"], p["deg"], p["W"], p["rows"], supports=p["supports"])
    A = O.assemble_A(p["cloud"], p["kind"], p["param"], p["deg"], supports=p["supports"])
    u, c = O.solve_direct(K, A, p["q"])
    return rel(u, g["vals"]), u, K


def _backward_error(K, c, q):
    b = np.concatenate([q, np.zeros(K.shape[0] - q.shape[0])])
    return np.abs(K @ c - b).max() / (np.abs(K) @ np.abs(c) + np.abs(b)).max()


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_solve_matches_reference(name, precision):
    """vals within 1e-10 (FP64 path) / 1e-8 (FP32 LU + FP64 GMRES) of the reference, or within 3x the
    oracle's own distance to the reference where that floor is larger."""
    import updes_gb300 as U
    g = load(name)
    case = case_of(g)
    p = oracle_problem(case)
    floor, u_or, K = _floor(g, p)
    cl, sol = solve_case(case, precision)
    tol = (1e-10 if precision == "fp64" else 1e-8)
    err = rel(sol.vals, g["vals"])
    assert err <= max(tol, 3 * floor), (err, floor, U.LAST_INFO)
    assert rel(sol.vals, u_or) <= max(tol, 3 * floor)
    # coefficients: as backward-stable as the reference's own on the oracle's K (coefficients of these
    # ill-conditioned systems are far less determined than vals, so they are compared through the residual)
    assert _backward_error(K, sol.coeffs, p["q"]) <= max(1e-13, 10 * _backward_error(K, g["coeffs"], p["q"]))
    assert U.LAST_INFO["converged"] == 1
    if precision == "fp32":
        assert U.LAST_INFO["fell_back"] == 0, U.LAST_INFO


def test_mat_materialises_reference_B():
    g = load("poisson_jitter_11x11")
    case = case_of(g)
    cl, sol = solve_case(case, "fp64")
    B = sol.mat.materialize()
    assert B.shape == (cl.N, cl.N)
    assert rel(B, g["B"]) < 1e-9


# Double-float assembly: every polyharmonic golden case, plus polyharmonic variants of the periodic and the
# Robin (Gaussian) cases so that every row kind is covered (r^3 and r^5).
DF_CASES = [nm for nm in C.CASES if C.CASES[nm]["rbf"][0] == "polyharmonic"] + [
    "periodic_imq_8x7@1", "gaussian_dnr_9x8@2", "thinplate_deg4_8x8@1"]


def _df_case(name):
    base, _, a = name.partition("@")
    case = dict(C.CASES[base])
    if a:
        case["rbf"] = ("polyharmonic", int(a))
    return case


def _assemble_df(dp):
    import torch
    lib = _lib.load()
    ld = int(lib.updes_matrix_ld(dp.n, 8))
    hi = torch.full((dp.n, ld), float("nan"), dtype=torch.float32, device="cuda")
    lo = torch.full((dp.n, ld), float("nan"), dtype=torch.float32, device="cuda")
    rowmax = torch.zeros(dp.n, dtype=torch.int32, device="cuda")
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    nb = ctypes.c_size_t()
    _lib.check(lib.updes_assemble_df_scratch(ctypes.byref(dp.c), ctypes.byref(nb)), "scratch")
    scratch = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    st = lib.updes_assemble_df(ctypes.byref(dp.c), hi.data_ptr(), lo.data_ptr(), ld, rowmax.data_ptr(),
                               flag.data_ptr(), scratch.data_ptr(), nb.value, dp.stream())
    torch.cuda.synchronize()
    return st, hi, lo, rowmax, flag, ld


@pytest.mark.parametrize("name", DF_CASES)
def test_df_assembly_matches_fp64(name):
    """The double-float planes hi + lo agree with the FP64 assembly to 2^-45 of each row's largest entry
    (the FP64 entries are themselves good to ~2^-50); padding columns are zero, the row maxima are those of
    |hi|, and no entry is flagged out of range."""
    case = _df_case(name)
    cl, dp, q = device_problem(case)
    K64, _, ld = assemble(dp)
    st, hi, lo, rowmax, flag, ld2 = _assemble_df(dp)
    _lib.check(st, "updes_assemble_df")
    assert ld2 == ld and int(flag.item()) == 0
    n = dp.n
    K = K64.cpu().numpy()
    H, L = hi.cpu().numpy(), lo.cpu().numpy()
    assert np.all(H[:, n:] == 0) and np.all(L[:, n:] == 0)
    D = H[:, :n].astype(np.float64) + L[:, :n].astype(np.float64)
    rmax = np.abs(K[:, :n]).max(axis=1)
    err = np.abs(D - K[:, :n]).max(axis=1)
    assert np.all(err <= 2.0 ** -45 * rmax), (err / rmax).max()
    assert np.all(np.abs(L[:, :n]) <= np.spacing(np.abs(H[:, :n])))  # normalised pairs
    want = np.abs(H[:, :n]).max(axis=1).astype(np.float32).view(np.int32)
    assert np.array_equal(rowmax.cpu().numpy(), want)


def test_df_assembly_rejects_other_kernels():
    cl, dp, q = device_problem(C.CASES["gaussian_dnr_9x8"])
    st = _assemble_df(dp)[0]
    assert st == _lib.ERR_UNSUPPORTED

def _rand_system(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 0.5 * np.eye(n)
    return A


@pytest.mark.parametrize("n", [1, 7, 64, 65, 200, 513])
@pytest.mark.parametrize("precision", [0, 1])
def test_lu_solve_random(n, precision):
    import torch
    lib = _lib.load()
    A = _rand_system(n, n)
    ld = int(lib.updes_matrix_ld(n, 8))
    Ad = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Ad[:, :n] = torch.as_tensor(A)
    F = torch.zeros((n, ld), dtype=torch.float32, device="cuda") if precision else None
    piv = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    nb = ctypes.c_size_t()
    _lib.check(lib.updes_lu_workspace(n, precision, ctypes.byref(nb)), "ws")
    ws = torch.empty(nb.value + 8 * n * 4 + 1024, dtype=torch.uint8, device="cuda")
    info = ctypes.c_int32(-1)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.updes_lu_factor(n, Ad.data_ptr(), ld, precision, F.data_ptr() if precision else None,
                                   ld if precision else 0, piv.data_ptr(), ws.data_ptr(), ws.numel(),
                                   ctypes.byref(info), s), "factor")
    assert info.value == 0
    Fp = F if precision else Ad
    # pivots follow LAPACK's choice (max |a|, first on ties) in the FP64 path
    if precision == 0:
        import scipy.linalg as sla
        lu, pv = sla.lu_factor(A)
        assert np.array_equal(piv[:n].cpu().numpy(), pv)
        assert np.allclose(Ad[:, :n].cpu().numpy(), lu, rtol=1e-10, atol=1e-10)
    rng = np.random.default_rng(1)
    B = rng.standard_normal((n, 3))
    for trans in (0, 1):
        Bd = torch.as_tensor(B.copy(), device="cuda")
        _lib.check(lib.updes_lu_solve(n, Fp.data_ptr(), ld, precision, piv.data_ptr(), Bd.data_ptr(), 3, 3, trans,
                                      ws.data_ptr(), ws.numel(), s), "solve")
        X = Bd.cpu().numpy()
        want = np.linalg.solve(A.T if trans else A, B)
        tol = 1e-10 if precision == 0 else 1e-3
        assert rel(X, want) < tol, (trans, rel(X, want))


def test_lu_reports_singular_pivot():
    import torch
    lib = _lib.load()
    n = 96
    A = _rand_system(n, 5)
    A[:, 17] = 0.0
    ld = int(lib.updes_matrix_ld(n, 8))
    Ad = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Ad[:, :n] = torch.as_tensor(A)
    piv = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    nb = ctypes.c_size_t()
    lib.updes_lu_workspace(n, 0, ctypes.byref(nb))
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    info = ctypes.c_int32(0)
    st = lib.updes_lu_factor(n, Ad.data_ptr(), ld, 0, None, 0, piv.data_ptr(), ws.data_ptr(), ws.numel(),
                             ctypes.byref(info), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0 and info.value == 18


def test_residual_kernel():
    import torch
    lib = _lib.load()
    n = 300
    A = _rand_system(n, 9)
    ld = int(lib.updes_matrix_ld(n, 8))
    Ad = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Ad[:, :n] = torch.as_tensor(A)
    rng = np.random.default_rng(2)
    x, b = rng.standard_normal(n), rng.standard_normal(n)
    xd, bd = torch.as_tensor(x, device="cuda"), torch.as_tensor(b, device="cuda")
    r = torch.empty(n, dtype=torch.float64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for trans in (0, 1):
        _lib.check(lib.updes_residual(n, Ad.data_ptr(), ld, xd.data_ptr(), bd.data_ptr(), r.data_ptr(), trans, s), "r")
        want = b - (A.T if trans else A) @ x
        assert rel(r.cpu().numpy(), want) < 1e-13


def _factor_both(n, seed):
    import torch
    lib = _lib.load()
    A = _rand_system(n, seed)
    ld = int(lib.updes_matrix_ld(n, 8))
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {}
    for precision in (0, 1):
        Ad = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
        Ad[:, :n] = torch.as_tensor(A)
        F = torch.zeros((n, ld), dtype=torch.float32, device="cuda") if precision else Ad
        piv = torch.empty(2 * n, dtype=torch.int32, device="cuda")
        nb = ctypes.c_size_t()
        _lib.check(lib.updes_lu_workspace(n, precision, ctypes.byref(nb)), "ws")
        ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
        info = ctypes.c_int32(-1)
        _lib.check(lib.updes_lu_factor(n, Ad.data_ptr(), ld, precision, F.data_ptr() if precision else None,
                                       ld if precision else 0, piv.data_ptr(), ws.data_ptr(), ws.numel(),
                                       ctypes.byref(info), s), "factor")
        assert info.value == 0
        out[precision] = (F[:, :n].double().cpu().numpy(), piv[:n].cpu().numpy())
    return out


@pytest.mark.parametrize("n", [70, 300, 700])
def test_mixed_factorisation_backward_error(n):
    """P A = L U holds to FP32-rounding level, |P A - L U| <= 2^-22 (|L| |U|) entrywise, for the FP32
    factors of the mixed LU (tensor-core digit-product updates in a double-float trailing matrix)."""
    out = _factor_both(n, 100 + n)
    A = _rand_system(n, 100 + n)
    for precision, tol in ((1, 2.0 ** -22), (0, 2.0 ** -48)):
        F, piv = out[precision]
        perm = np.arange(n)
        for i, p in enumerate(piv):
            perm[[i, p]] = perm[[p, i]]
        L = np.tril(F, -1) + np.eye(n)
        U = np.triu(F)
        R = np.abs(A[perm] - L @ U)
        bound = tol * (np.abs(L) @ np.abs(U)) + 1e-300
        assert np.all(R <= bound), (precision, (R / bound).max())


def test_mixed_refinement_iterations_on_ill_conditioned_system():
    """The Poisson r^3 / degree-2 system at N = 3,600 (kappa(K) ~ 1e10): an FP32-accumulated LU
    (LAPACK sgetrf) needs ~100 GMRES iterations here, an LU whose trailing updates are accurate needs
    a handful.  The mixed path must stay in the second class, without falling back to FP64."""
    import updes_gb300 as U
    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    cl = U.SquareCloud(Nx=60, Ny=60, facet_types=facets, jitter=(0.2, 0))
    ustar = lambda c: np.sin(np.pi * c[0]) * np.sin(np.pi * c[1])
    op = lambda x, center, rbf, monomial, fields: U.nodal_laplacian(x, center, rbf, monomial)
    rhs = lambda x, centers, rbf, fields: -2 * np.pi ** 2 * np.sin(np.pi * x[0]) * np.sin(np.pi * x[1])
    s32 = U.pde_solver(op, rhs, cl, {f: ustar for f in facets}, U.polyharmonic, 2,
                       options=U.SolverOptions(precision="fp32"))
    info = dict(U.LAST_INFO)
    s64 = U.pde_solver(op, rhs, cl, {f: ustar for f in facets}, U.polyharmonic, 2,
                       options=U.SolverOptions(precision="fp64"))
    assert info["fell_back"] == 0 and info["converged"] == 1, info
    assert info["iters"] <= 12, info
    assert rel(s32.vals, s64.vals) < 1e-8


def test_factor_once_solve_many():
    """updes_factor + updes_solve_factored on 3 right-hand sides equals 3 fresh updes_solve calls, and
    pde_solver reuses its factors when only the boundary values change."""
    import torch

    import updes_gb300 as U
    from gpu_helpers import device_problem
    lib = _lib.load()
    g = load("readme_laplace_30x20")
    case = case_of(g)
    cl, dp, q = device_problem(case)
    rng = np.random.default_rng(3)
    Q = np.stack([q, q + rng.standard_normal(q.shape) * 0.1, 2 * q], axis=1)  # N x 3
    opts = U.SolverOptions(precision="fp32")
    co = opts.c_opts()
    nb = ctypes.c_size_t()
    _lib.check(lib.updes_solve_workspace(ctypes.byref(dp.c), ctypes.byref(co), ctypes.byref(nb)), "ws")
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    info = _lib.SolveInfo()
    _lib.check(lib.updes_factor(ctypes.byref(dp.c), ctypes.byref(co), ctypes.byref(info), ws.data_ptr(), ws.numel(),
                                dp.stream()), "factor")
    Qd = torch.as_tensor(Q, device="cuda").contiguous()
    Cd = torch.empty((dp.n, 3), dtype=torch.float64, device="cuda")
    Vd = torch.empty((dp.N, 3), dtype=torch.float64, device="cuda")
    _lib.check(lib.updes_solve_factored(ctypes.byref(dp.c), 3, Qd.data_ptr(), 3, Cd.data_ptr(), 3, Vd.data_ptr(), 3,
                                        ctypes.byref(co), ctypes.byref(info), ws.data_ptr(), ws.numel(), dp.stream()),
               "solve_factored")
    for j in range(3):
        c1, v1, _ = U.operators.solve_device(dp, Q[:, j], U.SolverOptions(precision="fp32", reuse_factorization=False))
        assert rel(Vd[:, j].cpu().numpy(), v1.cpu().numpy()) < 1e-11
        assert rel(Cd[:, j].cpu().numpy(), c1.cpu().numpy()) < 1e-8
    # transparent reuse inside pde_solver
    from gpu_helpers import solve_case
    U.operators.free_factorizations()
    _, s1 = solve_case(case, "fp32")
    assert not U.LAST_INFO["reused_factors"]
    _, s2 = solve_case(case, "fp32")
    assert U.LAST_INFO["reused_factors"]
    assert rel(s2.vals, s1.vals) < 1e-12
    assert rel(s1.vals, g["vals"]) < 1e-8


@pytest.mark.parametrize("name", list(C.LOCAL_CASES))
def test_local_support_mat_and_coefficients(name):
    """Local supports through the rest of the solve's outputs: the materialised B against the reference's,
    core_compute_coefficients (A with local supports) against the oracle, and the batched evaluation, which
    does not take local supports, refusing them."""
    import torch

    import updes_gb300 as U
    from gpu_helpers import rbf_callable
    g = load(name)
    case = case_of(g)
    p = oracle_problem(case)
    cl, sol = solve_case(case, "fp64")
    assert rel(sol.mat.materialize(), g["B"]) < 1e-8
    f = np.sin(3 * cl.sorted_nodes[:, 0]) + cl.sorted_nodes[:, 1]
    got = U.compute_coefficients(f, cl, rbf_callable(case), case["max_degree"])
    want = O.field_coefficients(p["cloud"], p["kind"], p["param"], p["deg"], f, supports=p["supports"])
    A = O.assemble_A(p["cloud"], p["kind"], p["param"], p["deg"], supports=p["supports"])
    assert np.abs(A @ got - np.concatenate([f, np.zeros(dp_M(case))])).max() <= 1e-12 * np.abs(A).max() * max(
        np.abs(got).max(), 1.0)
    assert rel(A[:cl.N] @ got, A[:cl.N] @ want) < 1e-10
    _, dp, _ = device_problem(case)
    C_ = torch.zeros((dp.n, 2), dtype=torch.float64, device="cuda")
    V = torch.zeros((dp.N, 2), dtype=torch.float64, device="cuda")
    st = _lib.load().updes_eval_values_batch(ctypes.byref(dp.c), 2, C_.data_ptr(), 2, V.data_ptr(), 2, dp.stream())
    assert st == _lib.ERR_UNSUPPORTED


def dp_M(case):
    return O.nb_monomials(case["max_degree"])
