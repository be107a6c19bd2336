"""Helpers shared by the GPU tests: build a golden case's problem for the product."""
import ctypes

import numpy as np

import cases as C
import updes_gb300 as U
from test_host import _bcs, _diff_operator, product_cloud
from updes_gb300 import _lib


def rbf_callable(case):
    from functools import partial
    kind, p = case["rbf"]
    f = getattr(U, kind)
    return partial(f, **({"a": int(p)} if kind in ("polyharmonic", "thin_plate") else {"eps": p}))


def rhs_operator(case):
    name = case["rhs"]

    def f(x, centers=None, rbf=None, fields=None):
        if name == "value_over_dt":
            return U.value(x, fields[:, 0], centers, rbf) / C.ADV_DT
        return C.FUNCS[name](np, x[0], x[1])
    return f


def solve_case(case, precision, **kw):
    cl = product_cloud(case)
    fields = C.make_fields(case, cl.sorted_nodes)
    rf = C.make_rhs_field(case, cl.sorted_nodes)
    opts = U.SolverOptions(precision=precision, **kw)
    sol = U.pde_solver(_diff_operator(case["op"]), rhs_operator(case), cl, _bcs(case, cl), rbf_callable(case),
                       case["max_degree"], diff_args=None if fields is None else list(fields),
                       rhs_args=None if rf is None else [rf], options=opts)
    return cl, sol


def device_problem(case, compat=True):
    cl = product_cloud(case)
    fields = C.make_fields(case, cl.sorted_nodes)
    W, kind, bnodes, geom, q = U.operators.prepare(
        _diff_operator(case["op"]), rhs_operator(case), cl, _bcs(case, cl), rbf_callable(case), case["max_degree"],
        diff_args=None if fields is None else list(fields),
        rhs_args=None if C.make_rhs_field(case, cl.sorted_nodes) is None else [C.make_rhs_field(case, cl.sorted_nodes)],
        options=U.SolverOptions(compat_reference_quirks=compat))
    return cl, U.operators.DeviceProblem(cl, rbf_callable(case), case["max_degree"], W, kind, bnodes, geom), q


def assemble(dp, fp32=False):
    import torch
    lib = _lib.load()
    ld = int(lib.updes_matrix_ld(dp.n, 8))
    K64 = torch.full((dp.n, ld), float("nan"), dtype=torch.float64, device="cuda")
    K32 = torch.full((dp.n, ld), float("nan"), dtype=torch.float32, device="cuda") if fp32 else None
    st = lib.updes_assemble(ctypes.byref(dp.c), K64.data_ptr(), ld, K32.data_ptr() if fp32 else None,
                            ld if fp32 else 0, dp.stream())
    _lib.check(st, "updes_assemble")
    torch.cuda.synchronize()
    return K64, K32, ld


def lu_factor_random(n, precision, seed):
    """LU (updes_lu_factor) of a random n x n matrix + 0.5 I; returns (A, factors, ld, piv, workspace, stream)."""
    import torch
    lib = _lib.load()
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 0.5 * np.eye(n)
    ld = int(lib.updes_matrix_ld(n, 8))
    Ad = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Ad[:, :n] = torch.as_tensor(A)
    F = torch.zeros((n, ld), dtype=torch.float32, device="cuda") if precision else Ad
    piv = torch.empty(2 * n, dtype=torch.int32, device="cuda")
    nb = ctypes.c_size_t()
    _lib.check(lib.updes_lu_workspace(n, precision, ctypes.byref(nb)), "updes_lu_workspace")
    ws = torch.empty(nb.value + 8 * n * 4 + 1024, dtype=torch.uint8, device="cuda")
    info = ctypes.c_int32(-1)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(lib.updes_lu_factor(n, Ad.data_ptr(), ld, precision, F.data_ptr() if precision else None,
                                   ld if precision else 0, piv.data_ptr(), ws.data_ptr(), ws.numel(),
                                   ctypes.byref(info), s), "updes_lu_factor")
    assert info.value == 0
    return A, F, ld, piv, ws, s
