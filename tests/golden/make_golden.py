"""Generate the golden fixtures by running the reference (Updes 1.0.3) itself.

Usage (needs the Updes source tree; JAX is replaced by ``ref_shim``):

    python tests/golden/make_golden.py <path of the Updes source tree> [case ...]

For every case in ``cases.CASES`` this builds the reference ``SquareCloud``
(coordinates injected, so no RNG is shared), calls the reference's own
``pde_solver_jit`` and its assembly functions (``assemble_op_Phi_P``,
``assemble_bd_Phi_P``, ``assemble_A``, ``assemble_q``), and stores inputs and
outputs in ``tests/golden/<case>.npz``.  It also differentiates the reference
solve (reverse mode, through inv/GEMM/QR) for the boundary-control adjoint case,
runs the reference's ``pde_multi_solver`` on the two-field cases of
``cases.MULTI_CASES``, and reads the synthetic mesh of ``make_msh.py`` with the
reference's ``GmshCloud`` (solving ``cases.GMSH_CASE`` on it), and runs the reference's field helpers
(``integrate_field``, ``interpolate_field``, ``gradient_vals_vec``, the grid finite differences) on the
``cases.FIELD_*`` problems.
"""
from __future__ import annotations

import json
import os
import sys
import time
from functools import partial

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(1, os.path.dirname(os.path.dirname(HERE)))  # the product, for its GmshCloud check
import ref_shim  # noqa: E402

ref_shim.install()
import torch  # noqa: E402

import cases as C  # noqa: E402


def load_reference(path):
    sys.path.insert(0, path)
    import updes  # noqa: F401
    return updes


def build(updes, case):
    import jax.numpy as jnp
    coords = C.grid_coords(case)

    class InjectedCloud(updes.SquareCloud):
        def define_node_coordinates(self, noise_key):
            self.nodes = {g: torch.tensor(coords[g]) for g in range(self.N)}

    cloud = InjectedCloud(Nx=case["Nx"], Ny=case["Ny"], facet_types=dict(case["facets"]),
                          support_size=case.get("support", "max"))
    kind, param = case["rbf"]
    rbf = {"polyharmonic": lambda p: partial(updes.polyharmonic, a=int(p)),
           "gaussian": lambda p: partial(updes.gaussian, eps=p),
           "multiquadric": lambda p: partial(updes.multiquadric, eps=p),
           "inverse_multiquadric": lambda p: partial(updes.inverse_multiquadric, eps=p),
           "thin_plate": lambda p: partial(updes.thin_plate, a=int(p))}[kind](param)
    op = case["op"]

    def diff_operator(x, center=None, rbf=None, monomial=None, fields=None):
        val = updes.nodal_value(x, center, rbf, monomial)
        grad = updes.nodal_gradient(x, center, rbf, monomial)
        lap = updes.nodal_laplacian(x, center, rbf, monomial)
        if op == "laplacian":
            return lap
        if op == "advdiff":
            return val / C.ADV_DT + jnp.dot(jnp.array(C.ADV_VEL), grad) - C.ADV_K * lap
        if op == "kgrad":
            return fields[0] * lap + fields[1] * grad[0] + fields[2] * grad[1]
        if op == "darcy":
            return updes.nodal_div_grad(x, center, rbf, monomial, (fields[0], fields[0])) + fields[1] * val
        if op == "helmholtz_x":
            return lap + (1.0 + x[0] * x[1]) * val
        raise ValueError(op)

    rhs = case["rhs"]

    def rhs_operator(x, centers=None, rbf=None, fields=None):
        if rhs == "value_over_dt":
            return updes.value(x, fields[:, 0], centers, rbf) / C.ADV_DT
        return C.FUNCS[rhs](jnp, x[0], x[1])

    def bc_fn(name):
        return lambda coord: C.FUNCS[name](jnp, coord[0], coord[1])

    bcs = {}
    for f, spec in case["bc"].items():
        bcs[f] = (bc_fn(spec[0]), bc_fn(spec[1])) if isinstance(spec, tuple) else bc_fn(spec)
    nodes = np.asarray(cloud.sorted_nodes)
    fields = C.make_fields(case, nodes)
    diff_args = None if fields is None else [torch.tensor(f) for f in fields]
    rf = C.make_rhs_field(case, nodes)
    rhs_args = None if rf is None else [torch.tensor(rf)]
    return cloud, rbf, diff_operator, rhs_operator, bcs, diff_args, rhs_args


def run_case(updes, name, case):
    t0 = time.time()
    cloud, rbf, dop, rop, bcs, diff_args, rhs_args = build(updes, case)
    sol = updes.pde_solver_jit(diff_operator=dop, rhs_operator=rop, cloud=cloud, boundary_conditions=bcs,
                               rbf=rbf, max_degree=case["max_degree"], diff_args=diff_args, rhs_args=rhs_args)
    M = updes.compute_nb_monomials(case["max_degree"], 2)
    bcs_arr = updes.boundary_conditions_func_to_arr(bcs, cloud)
    robin, bcs2 = updes.duplicate_robin_coeffs(bcs_arr, cloud)
    bcs2 = updes.zerofy_periodic_cond(bcs2, cloud)
    opPhi, opP = updes.assemble_op_Phi_P(dop, cloud, rbf, M, diff_args)
    bdPhi, bdP = updes.assemble_bd_Phi_P(cloud, rbf, M, robin)
    A = updes.assemble_A(cloud, rbf, M)
    q = updes.assemble_q(rop, bcs2, cloud, rbf, M, rhs_args)
    npy = lambda t: np.asarray(t.detach() if isinstance(t, torch.Tensor) else t, dtype=np.float64)
    diffMat = np.concatenate([np.concatenate([npy(opPhi), npy(opP)], 1),
                              np.concatenate([npy(bdPhi), npy(bdP)], 1)], 0)
    A = npy(A)
    N = cloud.N
    out = dict(
        case=json.dumps(case),
        coords=C.grid_coords(case),
        sorted_nodes=npy(cloud.sorted_nodes),
        counts=np.array([cloud.N, cloud.Ni, cloud.Nd, cloud.Nn, cloud.Nr, sum(cloud.Np)], np.int64),
        facet_nodes=json.dumps({f: [int(i) for i in v] for f, v in cloud.facet_nodes.items()}),
        sorted_outward_normals=npy(getattr(cloud, "sorted_outward_normals", torch.zeros(0, 2))),
        robin=json.dumps({int(k): float(v) for k, v in robin.items()}),
        q=npy(q), vals=npy(sol.vals), coeffs=npy(sol.coeffs),
        diffMat_rowsum=diffMat.sum(1), diffMat_rowabs=np.abs(diffMat).sum(1),
        A_rowsum=A.sum(1), A_rowabs=np.abs(A).sum(1),
    )
    if case.get("support") is not None:
        out["sorted_local_supports"] = np.asarray(npy(cloud.sorted_local_supports), dtype=np.int64)
    if diff_args is not None:
        out["fields"] = np.stack([npy(f) for f in diff_args])
    if rhs_args is not None:
        out["rhs_field"] = npy(rhs_args[0])
    if N <= C.FULL_MATRIX_MAX_N:
        out.update(diffMat=diffMat, A=A, B=npy(sol.mat))
    else:
        rows = np.arange(0, N, C.ROW_STRIDE)
        out.update(diffMat_rows=rows, diffMat_sub=diffMat[rows], A_sub=A[rows],
                   B_sub=npy(sol.mat)[rows])
    # field operators on the solution (updes/operators.py:149-187)
    out["grad_at_nodes"] = npy(updes.gradient_vec(cloud.sorted_nodes, sol.coeffs, cloud.sorted_nodes, rbf))
    out["value_at_nodes"] = npy(updes.value_vec(cloud.sorted_nodes, sol.coeffs, cloud.sorted_nodes, rbf))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: N={N} n={N + M} {time.time() - t0:.1f}s")


def run_adjoint(updes, name=None):
    """Reverse-mode gradient through the reference solve (inv → GEMM → QR → inv)."""
    import jax.numpy as jnp
    name = name or C.ADJOINT_CASE
    case = C.CASES.get(name) or C.LOCAL_CASES[name]
    cloud, rbf, dop, rop, bcs, diff_args, rhs_args = build(updes, case)
    north = cloud.facet_nodes["North"]
    c0 = torch.tensor(C.adjoint_control(len(north)), requires_grad=True)
    fields = [f.clone().requires_grad_(True) for f in diff_args]
    nodes = cloud.sorted_nodes
    ut = C.adjoint_target(jnp, nodes[:, 0], nodes[:, 1])
    bcs = updes.boundary_conditions_func_to_arr(bcs, cloud)
    bcs["North"] = c0
    sol = updes.pde_solver(diff_operator=dop, rhs_operator=rop, cloud=cloud, boundary_conditions=bcs,
                           rbf=rbf, max_degree=case["max_degree"], diff_args=fields, rhs_args=None)
    Ni = cloud.Ni
    J = torch.mean((sol.vals[:Ni] - ut[:Ni]) ** 2) + C.ADJOINT_REG * torch.sum(c0 ** 2)
    J.backward()
    out_name = "adjoint_kgrad_10x10" if name == C.ADJOINT_CASE else f"adjoint_{name}"
    np.savez_compressed(os.path.join(HERE, f"{out_name}.npz"),
                        control=c0.detach().numpy(), J=np.array(float(J)),
                        dJ_dc=c0.grad.numpy(), dJ_dfields=np.stack([f.grad.numpy() for f in fields]),
                        vals=sol.vals.detach().numpy())
    print("adjoint: J =", float(J))


def run_multi(updes, name, case):
    """The reference's own pde_multi_solver (updes/operators.py:686-771) on a two-field system."""
    t0 = time.time()
    coords = C.grid_coords(case)

    class InjectedCloud(updes.SquareCloud):
        def define_node_coordinates(self, noise_key):
            self.nodes = {g: torch.tensor(coords[g]) for g in range(self.N)}

    cloud = InjectedCloud(Nx=case["Nx"], Ny=case["Ny"], facet_types=dict(case["facets"]), support_size="max")
    rbf = partial(updes.polyharmonic, a=int(case["rbf"][1]))
    if case["kind"] == "grayscott":
        def dop(x, center=None, rbf=None, monomial=None, fields=None):
            return updes.nodal_value(x, center, rbf, monomial)

        def rop_u(x, centers=None, rbf=None, fields=None):
            u_old, v_t = fields[:, 0], fields[:, 1]
            u, v = updes.value(x, u_old, centers, rbf), updes.value(x, v_t, centers, rbf)
            return C.GS_DU * updes.laplacian(x, u_old, centers, rbf) - u * v ** 2 + C.GS_F * (1 - u)

        def rop_v(x, centers=None, rbf=None, fields=None):
            u_t, v_old = fields[:, 0], fields[:, 1]
            u, v = updes.value(x, u_t, centers, rbf), updes.value(x, v_old, centers, rbf)
            return C.GS_DV * updes.laplacian(x, v_old, centers, rbf) + u * v ** 2 - (C.GS_F + C.GS_K) * v
        dops, rops = [dop, dop], [rop_u, rop_v]
    else:
        def dop(x, center=None, rbf=None, monomial=None, fields=None):
            val = updes.nodal_value(x, center, rbf, monomial)
            grad = updes.nodal_gradient(x, center, rbf, monomial)
            return val / C.BURGERS_DT + fields[0] * grad[0] + fields[1] * grad[1]

        def rop_u(x, centers=None, rbf=None, fields=None):
            return updes.value(x, fields[:, 0], centers, rbf) / C.BURGERS_DT

        def rop_v(x, centers=None, rbf=None, fields=None):
            return updes.value(x, fields[:, 1], centers, rbf) / C.BURGERS_DT
        dops, rops = [dop, dop], [rop_u, rop_v]
    zero = lambda c: 0.0 * c[0]
    bcs = {f: zero for f in case["facets"]}
    u0, v0 = C.multi_initial(case, np.asarray(cloud.sorted_nodes))
    prev = [torch.tensor(u0), torch.tensor(v0)]
    sols = updes.pde_multi_solver(diff_operators=dops, rhs_operators=rops, cloud=cloud,
                                  boundary_conditions=[dict(bcs), dict(bcs)], rbf=rbf,
                                  max_degree=case["max_degree"], nb_iters=case["nb_iters"], tol=1e-10,
                                  diff_args=[list(prev), list(prev)], rhs_args=[list(prev), list(prev)])
    npy = lambda t: np.asarray(t.detach() if isinstance(t, torch.Tensor) else t, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), case=json.dumps(case), coords=coords,
                        sorted_nodes=npy(cloud.sorted_nodes), u0=u0, v0=v0,
                        vals=np.stack([npy(s.vals) for s in sols]), coeffs=np.stack([npy(s.coeffs) for s in sols]))
    print(f"{name}: N={cloud.N} {time.time() - t0:.1f}s")


def run_gmsh(updes):
    """The reference's GmshCloud on the synthetic mesh and its pde_solver_jit on that cloud."""
    import jax.numpy as jnp
    t0 = time.time()
    case = C.GMSH_CASE
    cloud = updes.GmshCloud(filename=os.path.join(HERE, case["mesh"]), facet_types=dict(case["facets"]),
                            support_size="max")
    rbf = partial(updes.polyharmonic, a=int(case["rbf"][1]))

    def dop(x, center=None, rbf=None, monomial=None, fields=None):
        return updes.nodal_laplacian(x, center, rbf, monomial)

    def rop(x, centers=None, rbf=None, fields=None):
        return C.FUNCS[case["rhs"]](jnp, x[0], x[1])

    def bc_fn(name):
        return lambda coord: C.FUNCS[name](jnp, coord[0], coord[1])
    bcs = {f: (bc_fn(v[0]), bc_fn(v[1])) if isinstance(v, tuple) else bc_fn(v) for f, v in case["bc"].items()}
    sol = updes.pde_solver_jit(diff_operator=dop, rhs_operator=rop, cloud=cloud, boundary_conditions=bcs, rbf=rbf,
                               max_degree=case["max_degree"])
    npy = lambda t: np.asarray(t.detach() if isinstance(t, torch.Tensor) else t, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "gmsh_dshape.npz"), case=json.dumps(case),
                        sorted_nodes=npy(cloud.sorted_nodes), sorted_outward_normals=npy(cloud.sorted_outward_normals),
                        counts=np.array([cloud.N, cloud.Ni, cloud.Nd, cloud.Nn, cloud.Nr], np.int64),
                        facet_nodes=json.dumps({f: [int(i) for i in v] for f, v in cloud.facet_nodes.items()}),
                        node_types=json.dumps({int(k): v for k, v in cloud.node_types.items()}),
                        renumbering=json.dumps({int(k): int(v) for k, v in cloud.renumbering_map.items()}),
                        vals=npy(sol.vals), coeffs=npy(sol.coeffs))
    print(f"gmsh_dshape: N={cloud.N} {time.time() - t0:.1f}s")


def run_ref_fixture(updes, ref_path):
    """The reference's own unit test problem (updes/tests/test_operators.py:26-103): its GmshCloud on its mesh
    fixture (updes/tests/data/mesh.msh, every facet Neumann), Gaussian eps = 10, degree 1, operator
    nodal_value, rhs 12, zero Neumann values; the solution is the constant 12, whose gradient and divergence
    the reference test checks at atol 1e-2.  Stores the reference's cloud (so the GPU test can solve on it
    without the mesh file) and its vals, coeffs, gradients and divergences; the product's GmshCloud reads the
    same file here and must give the same cloud."""
    from updes_gb300.cloud import GmshCloud as ProductGmshCloud
    t0 = time.time()
    mesh = os.path.join(ref_path, "updes", "tests", "data", "mesh.msh")
    facets = {"Wall": "n", "Inflow": "n", "Outflow": "n", "Blowing": "n", "Suction": "n"}
    cloud = updes.GmshCloud(filename=mesh, facet_types=dict(facets))
    rbf = partial(updes.gaussian, eps=10.0)

    def dop(x, center=None, rbf=None, monomial=None, fields=None):
        return updes.nodal_value(x, center, rbf, monomial)

    def rop(x, centers=None, rbf=None, fields=None):
        return 12.0

    zero = lambda c: 0.0
    bcs = {f: zero for f in facets}
    sol = updes.pde_solver(diff_operator=dop, rhs_operator=rop, cloud=cloud, boundary_conditions=bcs, rbf=rbf,
                           max_degree=1)
    npy = lambda t: np.asarray(t.detach() if isinstance(t, torch.Tensor) else t, dtype=np.float64)
    grads = npy(updes.gradient_vec(cloud.sorted_nodes, sol.coeffs, cloud.sorted_nodes, rbf))
    field_vec = torch.stack([sol.coeffs, sol.coeffs], dim=-1)
    divs = npy(updes.divergence_vec(cloud.sorted_nodes, field_vec, cloud.sorted_nodes, rbf))
    mine = ProductGmshCloud(mesh, facet_types=dict(facets))
    assert np.array_equal(mine.sorted_nodes, npy(cloud.sorted_nodes))
    assert mine.facet_nodes == {f: [int(i) for i in v] for f, v in cloud.facet_nodes.items()}
    assert np.allclose(mine.sorted_outward_normals, npy(cloud.sorted_outward_normals), rtol=0, atol=1e-12)
    np.savez_compressed(os.path.join(HERE, "ref_test_operators_mesh.npz"), facets=json.dumps(facets),
                        sorted_nodes=npy(cloud.sorted_nodes), sorted_outward_normals=npy(cloud.sorted_outward_normals),
                        counts=np.array([cloud.N, cloud.Ni, cloud.Nd, cloud.Nn, cloud.Nr], np.int64),
                        facet_nodes=json.dumps({f: [int(i) for i in v] for f, v in cloud.facet_nodes.items()}),
                        node_types=json.dumps({int(k): v for k, v in cloud.node_types.items()}),
                        vals=npy(sol.vals), coeffs=npy(sol.coeffs), grads=grads, divs=divs,
                        product_cloud_checked=np.array(True))
    print(f"ref_test_operators_mesh: N={cloud.N} max |grad| {np.abs(grads).max():.2e} "
          f"max |div| {np.abs(divs).max():.2e} {time.time() - t0:.1f}s")


def run_fields(updes):
    """Field helpers: the reference's integrate_field on coefficients from its own interpolation solve,
    gradient_vals_vec / laplacian_vals_vec at a few points, interpolate_field between two numberings of one
    grid, apply_neumann_conditions, cartesian_gradient_vec and enforce_cartesian_gradient_neumann on a
    jittered grid with Neumann facets.  Writes tests/golden/fields_helpers.npz."""
    import jax.numpy as jnp
    t0 = time.time()
    npy = lambda t: np.asarray(t.detach() if isinstance(t, torch.Tensor) else t, dtype=np.float64)
    out = {}

    def injected(Nx, Ny, facets, coords, support="max"):
        class InjectedCloud(updes.SquareCloud):
            def define_node_coordinates(self, noise_key):
                self.nodes = {g: torch.tensor(coords[g]) for g in range(self.N)}
        return InjectedCloud(Nx=Nx, Ny=Ny, facet_types=dict(facets), support_size=support)

    for name, fc in C.FIELD_INTEGRAL_CASES.items():
        coords = C.grid_coords(fc)
        cloud = injected(fc["Nx"], fc["Ny"], fc["facets"], coords)
        rbf = partial(updes.polyharmonic, a=int(fc["rbf"][1]))
        X = npy(cloud.sorted_nodes)
        s = C.field_s(X)
        coeffs = updes.get_field_coefficients(jnp.asarray(s), cloud, rbf, fc["max_degree"])
        val = updes.integrate_field(coeffs, cloud, rbf, fc["max_degree"])
        P = jnp.asarray(C.FIELD_EVAL_POINTS)
        gv = updes.gradient_vals_vec(P, jnp.asarray(s), cloud, rbf, fc["max_degree"])
        lv = updes.laplacian_vals_vec(P, jnp.asarray(s), cloud, rbf, fc["max_degree"])
        out.update({f"{name}_field": s, f"{name}_coeffs": npy(coeffs), f"{name}_integral": np.float64(npy(val)),
                    f"{name}_gradient_vals": npy(gv), f"{name}_laplacian_vals": npy(lv),
                    f"{name}_sorted_nodes": X})
        print(f"{name}: integral {float(npy(val)):.12f} (pi/12 = {np.pi / 12:.12f})")

    ic = C.FIELD_INTERP_CASE
    N = ic["Nx"] * ic["Ny"]
    c1 = updes.SquareCloud(Nx=ic["Nx"], Ny=ic["Ny"], facet_types=dict(ic["facets1"]), support_size=N - 1)
    c2 = updes.SquareCloud(Nx=ic["Nx"], Ny=ic["Ny"], facet_types=dict(ic["facets2"]), support_size=N - 1)
    field = jnp.arange(0, c1.N)
    out["interp_field"] = npy(field)
    out["interp_result"] = npy(updes.interpolate_field(field, c1, c2))

    fd = C.FIELD_FD_CASE
    coords = C.grid_coords(fd)
    cloud = injected(fd["Nx"], fd["Ny"], fd["facets"], coords)
    X = npy(cloud.sorted_nodes)
    f = np.sin(2.0 * X[:, 0]) + X[:, 1] ** 2 + 0.3 * X[:, 0] * X[:, 1]
    bcs = {k: None for k in fd["facets"]}
    out["fd_field"] = f
    out["fd_sorted_nodes"] = X
    out["fd_neumann"] = npy(updes.apply_neumann_conditions(jnp.asarray(f), bcs, cloud))
    grads = updes.cartesian_gradient_vec(range(cloud.N), jnp.asarray(f), cloud)
    out["fd_cartesian_gradient"] = npy(grads)
    out["fd_enforced"] = npy(updes.enforce_cartesian_gradient_neumann(jnp.asarray(f), grads, bcs, cloud))
    # the same on k-nearest supports (support_size an int)
    cloud = injected(fd["Nx"], fd["Ny"], fd["facets"], coords, support=C.FIELD_FD_SUPPORT)
    out["fdl_neumann"] = npy(updes.apply_neumann_conditions(jnp.asarray(f), bcs, cloud))
    grads = updes.cartesian_gradient_vec(range(cloud.N), jnp.asarray(f), cloud)
    out["fdl_cartesian_gradient"] = npy(grads)
    out["fdl_enforced"] = npy(updes.enforce_cartesian_gradient_neumann(jnp.asarray(f), grads, bcs, cloud))
    np.savez_compressed(os.path.join(HERE, "fields_helpers.npz"), **out)
    print(f"fields_helpers: {len(out)} arrays, {time.time() - t0:.1f}s")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <path of the Updes source tree> [case ...]")
    ref = sys.argv[1]
    updes = load_reference(ref)
    only = sys.argv[2:] or (list(C.CASES) + list(C.MULTI_CASES) + list(C.LOCAL_CASES)
                            + ["gmsh", "ref_fixture", "adjoint_local", "fields"])
    for name in only:
        if name == "adjoint":
            continue
        if name == "gmsh":
            run_gmsh(updes)
            continue
        if name == "ref_fixture":
            run_ref_fixture(updes, ref)
            continue
        if name == "fields":
            run_fields(updes)
            continue
        if name == "adjoint_local":
            run_adjoint(updes, C.LOCAL_ADJOINT_CASE)
            continue
        if name in C.MULTI_CASES:
            run_multi(updes, name, C.MULTI_CASES[name])
        elif name in C.LOCAL_CASES:
            run_case(updes, name, C.LOCAL_CASES[name])
        else:
            run_case(updes, name, C.CASES[name])
    if len(sys.argv) <= 2 or "adjoint" in sys.argv[2:]:
        run_adjoint(updes)
