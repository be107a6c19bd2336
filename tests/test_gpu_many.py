"""GPU: many independent systems in one call (updes_solve_many, pde_solver_many)."""
import numpy as np
import pytest

import cases as C
from gpu_helpers import rbf_callable, rhs_operator
from test_host import _bcs, _diff_operator, product_cloud
import updes_gb300 as U

pytestmark = pytest.mark.gpu


def _system(name):
    case = C.CASES[name]
    cl = product_cloud(case)
    fields = C.make_fields(case, cl.sorted_nodes)
    rf = C.make_rhs_field(case, cl.sorted_nodes)
    return dict(diff_operator=_diff_operator(case["op"]), rhs_operator=rhs_operator(case), cloud=cl,
                boundary_conditions=_bcs(case, cl), rbf=rbf_callable(case), max_degree=case["max_degree"],
                diff_args=None if fields is None else list(fields), rhs_args=None if rf is None else [rf])


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("streams", [1, 4])
def test_many_equals_one_by_one(precision, streams):
    """Every golden case (some twice) in one call: each result is bitwise the system solved alone."""
    names = list(C.CASES) + ["readme_laplace_30x20", "poisson_jitter_11x11"]
    systems = [_system(nm) for nm in names]
    opts = U.SolverOptions(precision=precision, reuse_factorization=False)
    many = U.pde_solver_many(systems, options=opts, streams=streams)
    assert len(many) == len(systems)
    for sysd, sol in zip(systems, many):
        one = U.pde_solver(options=opts, **sysd)
        assert np.array_equal(sol.vals, one.vals)
        assert np.array_equal(sol.coeffs, one.coeffs)
    infos = U.operators.LAST_MANY_INFO
    assert len(infos) == len(systems) and all(i["converged"] == 1 for i in infos)


def test_many_rejects_bad_arguments():
    from updes_gb300 import _lib
    import ctypes
    lib = _lib.load()
    nb = ctypes.c_size_t()
    assert lib.updes_solve_many_workspace(None, 1, None, 1, ctypes.byref(nb)) == _lib.ERR_INVALID
    assert lib.updes_solve_many(None, 0, None, None, None, None, None, None, 0, 1) == _lib.ERR_INVALID


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_many_uneven_clouds(precision):
    """Uneven clouds (100 to 2,025 nodes; Gaussian and r^5 kernels; Dirichlet, Neumann and Robin facets) on
    8 streams: systems of different sizes factor at the same time, a second call repeats the first bitwise,
    and each result is bitwise the system solved alone."""
    from updes_gb300 import workloads as WL
    systems = WL.uneven_clouds(24, seed=3)
    opts = U.SolverOptions(precision=precision, reuse_factorization=False)
    first = U.pde_solver_many(systems, options=opts, streams=8)
    many = U.pde_solver_many(systems, options=opts, streams=8)
    infos = U.operators.LAST_MANY_INFO
    assert all(i["converged"] == 1 for i in infos)
    for a, b in zip(first, many):
        assert np.array_equal(a.vals, b.vals)
    for k in (0, 1, 7, 23):
        one = U.pde_solver_jit(options=opts, **systems[k])
        assert np.array_equal(many[k].vals, one.vals)
        assert np.array_equal(many[k].coeffs, one.coeffs)
