"""GPU: many systems in one persistent launch (updes_solve_batched / pde_solver_batched).

* Every golden case, in both elimination precisions, against the reference's vals (the same bounds as the
  single-system solve: 1e-10 FP64, 1e-8 mixed, or 3x the oracle's own floor where that is larger).
* A slice of the uneven-cloud workload (Gaussian and r^5 systems of up to 45 x 45 nodes): the r^5 systems'
  vals against the oracle (within what FP64 determines), every system's backward error.
* Systems the batched launch does not take (local supports, n > 4096) are refused.
"""
import numpy as np
import pytest

import cases as C
import updes_gb300 as U
from golden_problem import case_of, load, oracle_problem
from gpu_helpers import rbf_callable, rhs_operator
from oracle import updes_np as O
from test_host import _bcs, _diff_operator, product_cloud
from updes_gb300 import _lib
from updes_gb300.batched import LAST_BATCHED_INFO, PanelTuner

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def _system(case):
    cl = product_cloud(case)
    fields = C.make_fields(case, cl.sorted_nodes)
    rf = C.make_rhs_field(case, cl.sorted_nodes)
    return dict(diff_operator=_diff_operator(case["op"]), rhs_operator=rhs_operator(case), cloud=cl,
                boundary_conditions=_bcs(case, cl), rbf=rbf_callable(case), max_degree=case["max_degree"],
                diff_args=None if fields is None else list(fields), rhs_args=None if rf is None else [rf])


def _floor(name):
    g = load(name)
    p = oracle_problem(case_of(g))
    K = O.assemble_K(p["cloud"], p["kind"], p["param"], p["deg"], p["W"], p["rows"])
    A = O.assemble_A(p["cloud"], p["kind"], p["param"], p["deg"])
    u, _ = O.solve_direct(K, A, p["q"])
    return rel(u, g["vals"])


@pytest.mark.parametrize("precision", ["fp64", "fp32", "auto"])
def test_golden_cases_in_one_launch(precision):
    names = list(C.CASES)
    systems = [_system(C.CASES[nm]) for nm in names]
    sols = U.pde_solver_batched(systems, precision=precision, tuner=PanelTuner(cache_path=None))
    for nm, sol, info in zip(names, sols, LAST_BATCHED_INFO):
        g = load(nm)
        tol = 1e-10 if precision == "fp64" else 1e-8
        err = rel(sol.vals, g["vals"])
        assert err <= max(tol, 3 * _floor(nm)), (nm, err, info)
        assert info["lu_info"] == 0, (nm, info)


def _oracle_solves(sysd):
    """The FP64 oracle's direct LU of one system's K, and the same with every entry of K moved by up to one
    ulp (seeded): the distance between the two is what FP64 determines of this system's vals."""
    W, kind, bnodes, geom, q = U.operators.prepare(sysd["diff_operator"], sysd["rhs_operator"], sysd["cloud"],
                                                   U.operators.boundary_conditions_func_to_arr(
                                                       sysd["boundary_conditions"], sysd["cloud"]),
                                                   sysd["rbf"], 2)
    cl = O.square_cloud(sysd["cloud"].Nx, sysd["cloud"].Ny, dict(sysd["cloud"].facet_types))
    cl.sorted_nodes = sysd["cloud"].sorted_nodes
    rows = O.BoundaryRows(kind=kind, i1=bnodes[:, 0], i2=bnodes[:, 1], n1=geom[:, 0:2], n2=geom[:, 2:4],
                          nP=geom[:, 4:6], beta=geom[:, 6])
    K = O.assemble_K(cl, "polyharmonic", 2, 2, W, rows)
    A = O.assemble_A(cl, "polyharmonic", 2, 2)
    u, _ = O.solve_direct(K, A, q)
    Kp = K * (1.0 + np.random.default_rng(7).uniform(-1.0, 1.0, K.shape) * 2.0 ** -53)
    up, _ = O.solve_direct(Kp, A, q)
    return u, rel(up, u)


def test_uneven_clouds_against_the_oracle_and_per_problem_fp64():
    """24 systems of the uneven-cloud workload (alternating Gaussian eps in [1, 5] and r^5, 100-2,025
    nodes, Dirichlet/Neumann/Robin facets) in one "auto" launch.  Every r^5 system reaches the refinement
    floor (32 unit roundoffs) and its vals lie within 1e-8, or 10x what FP64 determines (the distance
    between the oracle's LU of K and of K with its entries moved by an ulp) where that is larger, of the
    oracle's direct LU -- as do the per-problem FP64 solves'.  The Gaussian systems, too ill-conditioned for
    their vals to be compared, keep a backward error below 1e-12 (the FP64 relaunch threshold)."""
    from updes_gb300 import workloads as WL
    systems = WL.uneven_clouds(24, seed=3)
    ref = U.pde_solver_many(systems, options=U.SolverOptions(precision="fp64", reuse_factorization=False),
                            streams=4)
    got = U.pde_solver_batched(systems, precision="auto", tuner=PanelTuner(cache_path=None))
    infos = list(LAST_BATCHED_INFO)
    print("backward errors:", [f"{i['backward_error']:.1e}" for i in infos])
    for k in range(len(systems)):
        assert infos[k]["backward_error"] <= 1e-12, infos[k]
    for k in range(1, len(systems), 2):
        assert infos[k]["converged"] == 1, infos[k]
        u, floor = _oracle_solves(systems[k])
        eb, ef = rel(got[k].vals, u), rel(ref[k].vals, u)
        print(f"system {k} (N={systems[k]['cloud'].N}): batched {eb:.1e}, per-problem FP64 {ef:.1e}, "
              f"FP64 floor {floor:.1e}")
        assert eb <= max(1e-8, 10 * floor), (k, eb, floor)
        assert ef <= max(1e-8, 10 * floor), (k, ef, floor)


def test_systems_the_batched_launch_refuses():
    case = dict(C.LOCAL_CASES["poisson_local_12x12"])
    with pytest.raises(_lib.UpdesError) as ei:
        U.pde_solver_batched([_system(case)], tuner=None)
    assert ei.value.status == _lib.ERR_UNSUPPORTED
    from updes_gb300 import workloads as WL
    with pytest.raises(ValueError):
        U.pde_solver_batched([WL.poisson_manufactured(64)], tuner=None)  # n = 4,102
