"""Host-side logic (no GPU): cloud ordering, row descriptors, operator capture, C-ABI exports."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

import cases as C
import updes_gb300 as U
from golden_problem import case_of, load, oracle_problem
from oracle import updes_np as O
from updes_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = list(C.CASES)


def product_cloud(case):
    return U.SquareCloud(Nx=case["Nx"], Ny=case["Ny"], facet_types=dict(case["facets"]),
                         coords=C.grid_coords(case), support_size=case.get("support", "max"))


@pytest.mark.parametrize("name", NAMES)
def test_cloud_matches_reference(name):
    g = load(name)
    case = case_of(g)
    cl = product_cloud(case)
    assert np.array_equal(cl.sorted_nodes, g["sorted_nodes"])
    assert [cl.N, cl.Ni, cl.Nd, cl.Nn, cl.Nr, sum(cl.Np)] == g["counts"].tolist()
    assert cl.facet_nodes == json.loads(str(g["facet_nodes"]))
    assert np.array_equal(cl.sorted_outward_normals.reshape(-1, 2), g["sorted_outward_normals"].reshape(-1, 2))


def test_jitter_matches_case_generator():
    case = C.CASES["poisson_jitter_11x11"]
    a = U.SquareCloud(Nx=11, Ny=11, facet_types=dict(case["facets"]), jitter=case["jitter"])
    b = product_cloud(case)
    assert np.array_equal(a.sorted_nodes, b.sorted_nodes)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("compat", [True, False])
def test_boundary_rows_match_oracle(name, compat):
    g = load(name)
    case = case_of(g)
    p = oracle_problem(case, compat=compat)
    cl = product_cloud(case)
    rows = p["rows"]
    _, robin = U.operators._bc_values_and_betas(_bcs(case, cl), cl, compat)
    kind, nodes, geom = U.operators.boundary_rows(cl, robin, compat)
    assert np.array_equal(kind, rows.kind)
    assert np.array_equal(nodes[:, 0], rows.i1) and np.array_equal(nodes[:, 1], rows.i2)
    assert np.array_equal(geom[:, 0:2], rows.n1)
    per = rows.kind >= O.ROW_PD
    assert np.array_equal(geom[per, 2:4], rows.n2[per])
    assert np.array_equal(geom[:, 4:6], rows.nP)
    assert np.array_equal(geom[:, 6], rows.beta)


def _bcs(case, cl):
    out = {}
    for f, spec in case["bc"].items():
        fn = lambda name: (lambda x: C.FUNCS[name](np, x[0], x[1]))
        out[f] = (fn(spec[0]), fn(spec[1])) if isinstance(spec, tuple) else fn(spec)
    return out


def _diff_operator(op):
    """The golden cases' operators written against updes_gb300's nodal operators."""
    def f(x, center=None, rbf=None, monomial=None, fields=None):
        val = U.nodal_value(x, center, rbf, monomial)
        grad = U.nodal_gradient(x, center, rbf, monomial)
        lap = U.nodal_laplacian(x, center, rbf, monomial)
        if op == "laplacian":
            return lap
        if op == "advdiff":
            return val / C.ADV_DT + np.dot(np.array(C.ADV_VEL), grad) - C.ADV_K * lap
        if op == "kgrad":
            return fields[0] * lap + fields[1] * grad[0] + fields[2] * grad[1]
        if op == "darcy":
            return U.nodal_div_grad(x, center, rbf, monomial, (fields[0], fields[0])) + fields[1] * val
        if op == "helmholtz_x":
            return lap + (1.0 + x[0] * x[1]) * val
        raise ValueError(op)
    return f


@pytest.mark.parametrize("name", NAMES)
def test_operator_capture(name):
    g = load(name)
    case = case_of(g)
    cl = product_cloud(case)
    X = cl.sorted_nodes[:cl.Ni]
    fields = C.make_fields(case, cl.sorted_nodes)
    W = U.capture_operator(_diff_operator(case["op"]), X, U.polyharmonic,
                           None if fields is None else fields[:, :cl.Ni])
    ref = C.op_weights(case["op"], X[:, 0], X[:, 1], None if fields is None else fields[:, :cl.Ni])
    assert np.allclose(W, ref, rtol=1e-14, atol=1e-14)


def test_capture_rejects_nonlinear():
    X = np.random.default_rng(0).uniform(size=(5, 2))
    with pytest.raises(ValueError):
        U.capture_operator(lambda x, c, r, m, f: U.nodal_value(x, c, r, m) ** 2, X, U.polyharmonic, None)
    with pytest.raises(ValueError):
        U.capture_operator(lambda x, c, r, m, f: U.nodal_laplacian(x, c, r, m) + 1.0, X, U.polyharmonic, None)


def test_capture_per_node_fallback():
    """An operator that only works on one point at a time is captured node by node."""
    X = np.random.default_rng(0).uniform(size=(7, 2))

    def op(x, center, rbf, monomial, fields):
        assert np.asarray(x).shape == (2,)
        vel = np.array([x[1], -x[0]])
        return vel @ U.nodal_gradient(x, center, rbf, monomial) + U.nodal_laplacian(x, center, rbf, monomial)
    W = U.capture_operator(op, X, U.polyharmonic, None)
    assert np.allclose(W[:, 1], X[:, 1]) and np.allclose(W[:, 2], -X[:, 0]) and np.allclose(W[:, 3:], 1.0)


def test_rbf_spec():
    from functools import partial
    assert U.rbf_spec(U.polyharmonic) == (_lib.RBF_POLYHARMONIC, 1.0)
    assert U.rbf_spec(partial(U.polyharmonic, a=2)) == (_lib.RBF_POLYHARMONIC, 2.0)
    assert U.rbf_spec(partial(U.gaussian, eps=3.0)) == (_lib.RBF_GAUSSIAN, 3.0)
    with pytest.raises(ValueError):
        U.rbf_spec(lambda x, c: 1.0)
    with pytest.raises(ValueError):
        U.rbf_spec(partial(U.polyharmonic, a=1.5))


def test_nodal_numeric_matches_oracle():
    rng = np.random.default_rng(3)
    for kind, p in [("polyharmonic", 2), ("gaussian", 2.0), ("multiquadric", 1.5), ("inverse_multiquadric", 0.7),
                    ("thin_plate", 1)]:
        rbf = getattr(U, kind)
        from functools import partial
        rbf = partial(rbf, **({"a": p} if kind in ("polyharmonic", "thin_plate") else {"eps": p}))
        x, c = rng.uniform(size=2), rng.uniform(size=2)
        t = O.rbf_terms(kind, p, x[0] - c[0], x[1] - c[1])
        assert np.isclose(U.nodal_value(x, c, rbf), t[0], rtol=1e-13)
        assert np.allclose(U.nodal_gradient(x, c, rbf), [t[1], t[2]], rtol=1e-13)
        assert np.isclose(U.nodal_laplacian(x, c, rbf), t[3] + t[4], rtol=1e-13)
        assert np.isclose(rbf(x, c), t[0], rtol=1e-13)


def test_library_exports_every_declared_symbol():
    """The C-ABI library loads and exports every function include/updes_gb300.h declares."""
    if not os.path.exists(_lib.LIB_PATH):
        from updes_gb300 import build
        build.build()
    lib = _lib.load()
    header = open(os.path.join(ROOT, "include", "updes_gb300.h")).read()
    declared = set(re.findall(r"UPDES_API\s+[\w\s\*]+?\b(updes_\w+)\s*\(", header))
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(_lib.SIGNATURES), declared ^ set(_lib.SIGNATURES)
    assert lib.updes_version() >= 100
    assert lib.updes_status_string(_lib.ERR_SINGULAR).decode().startswith("singular")
    assert lib.updes_matrix_ld(22506, 8) == 22528


def test_invalid_arguments_rejected_without_gpu():
    """Argument validation runs before any CUDA call."""
    lib = _lib.load()
    p = _lib.Problem()
    p.N, p.Ni, p.M = 10, 4, 7  # invalid monomial count
    assert lib.updes_assemble(ctypes.byref(p), None, 0, None, 0, None) == _lib.ERR_INVALID
    nb = ctypes.c_size_t()
    assert lib.updes_lu_workspace(0, 0, ctypes.byref(nb)) == _lib.ERR_INVALID
    assert lib.updes_lu_workspace(100, 5, ctypes.byref(nb)) == _lib.ERR_INVALID
    assert lib.updes_lu_workspace(100, 1, ctypes.byref(nb)) == _lib.OK and nb.value > 0


@pytest.mark.parametrize("name", list(C.LOCAL_CASES))
def test_local_supports_match_reference(name):
    """SquareCloud(support_size=k): every node's support, as a set, equals the reference's BallTree result;
    GmshCloud takes the same path (updes/cloud.py:83-112)."""
    g = load(name)
    cl = product_cloud(case_of(g))
    ref = g["sorted_local_supports"]
    assert cl.sorted_local_supports.shape == ref.shape and cl.sorted_local_supports.dtype == np.int32
    assert all(set(a) == set(b) for a, b in zip(cl.sorted_local_supports.tolist(), ref.tolist()))


def test_support_size_edge_values():
    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    assert U.SquareCloud(Nx=5, Ny=4, facet_types=facets, support_size=20).sorted_local_supports is None
    assert U.SquareCloud(Nx=5, Ny=4, facet_types=facets, support_size="max").sorted_local_supports is None
    with pytest.raises(AssertionError):
        U.SquareCloud(Nx=5, Ny=4, facet_types=facets, support_size=21)
    with pytest.raises(ValueError):
        U.SquareCloud(Nx=5, Ny=4, facet_types=facets, support_size=1)
    with pytest.raises(ValueError):
        U.SquareCloud(Nx=5, Ny=4, facet_types=facets, support_size=2.5)


@pytest.mark.parametrize("name", NAMES)
def test_stacked_probes_equal_probes_one_by_one(name, monkeypatch):
    """The eight capture probes evaluated in one stacked call give the same weights, bit for bit, as the
    probes evaluated one at a time."""
    from updes_gb300 import operators as OPS
    g = load(name)
    case = case_of(g)
    cl = product_cloud(case)
    X = cl.sorted_nodes[:cl.Ni]
    fields = C.make_fields(case, cl.sorted_nodes)
    fl = None if fields is None else fields[:, :cl.Ni]
    op = _diff_operator(case["op"])
    stacked = U.capture_operator(op, X, U.polyharmonic, fl)
    monkeypatch.setattr(OPS, "_STACKED_PROBE_MAX_NODES", -1)
    assert np.array_equal(stacked, U.capture_operator(op, X, U.polyharmonic, fl))


def test_stacked_probe_falls_back_for_an_operator_that_mixes_probes(monkeypatch):
    """An operator that reduces over a primitive's whole value (here the mean of nodal_value, which is the
    value itself for one probe) mixes the stacked probes; the check against a separate evaluation catches it
    and the probes run one by one, giving the one-by-one weights."""
    from updes_gb300 import operators as OPS
    X = np.random.default_rng(1).uniform(size=(9, 2))
    op = lambda x, c, r, m, f: U.nodal_laplacian(x, c, r, m) + np.mean(U.nodal_value(x, c, r, m))
    calls = []
    orig = OPS.np.array_equal
    monkeypatch.setattr(OPS.np, "array_equal", lambda a, b: calls.append(orig(a, b)) or calls[-1])
    W = U.capture_operator(op, X, U.polyharmonic, None)
    assert calls == [False]
    assert np.allclose(W[:, 0], 1.0) and np.allclose(W[:, 1:3], 0.0) and np.allclose(W[:, 3:], 1.0)


def test_kernel_forms_of_r():
    from updes_gb300 import assembly as ASM
    r = np.array([0.0, 0.5, 2.0])
    assert np.allclose(ASM.polyharmonic_func(r, 1), r ** 3)
    assert np.allclose(ASM.gaussian_func(r, 2.0), np.exp(-(2.0 * r) ** 2))
    assert np.allclose(ASM.multiquadric_func(r, 1.5), np.sqrt(1 + (1.5 * r) ** 2))
    assert np.allclose(ASM.inv_multiquadric_func(r, 1.5), 1 / np.sqrt(1 + (1.5 * r) ** 2))
    assert np.allclose(ASM.thin_plate_func(r, 1), [0.0, np.log(0.5) * 0.25, np.log(2.0) * 4.0])
    assert ASM.make_nodal_rbf(np.array([0.0, 0.0]), np.array([3.0, 4.0]), lambda d: 2 * d) == 10.0


@pytest.mark.parametrize("kind,param", [("polyharmonic", 1), ("polyharmonic", 2), ("gaussian", 1.7),
                                        ("multiquadric", 0.8), ("inverse_multiquadric", 1.3), ("thin_plate", 1)])
def test_core_derivatives_match_central_differences(kind, param):
    """core_gradient_rbf / core_laplacian_rbf (the reference's grad and jacfwd(grad) of a kernel) against
    central differences of the kernel itself; the monomial versions likewise."""
    from functools import partial
    rbf = {"polyharmonic": partial(U.polyharmonic, a=param), "gaussian": partial(U.gaussian, eps=param),
           "multiquadric": partial(U.multiquadric, eps=param),
           "inverse_multiquadric": partial(U.inverse_multiquadric, eps=param),
           "thin_plate": partial(U.thin_plate, a=param)}[kind]
    x, c, h = np.array([0.31, 0.72]), np.array([0.55, 0.41]), 1e-4
    e = np.eye(2) * h
    g = U.core_gradient_rbf(rbf)(x, c)
    gfd = np.array([(rbf(x + e[i], c) - rbf(x - e[i], c)) / (2 * h) for i in range(2)])
    assert np.allclose(g, gfd, rtol=1e-6, atol=1e-9)
    H = U.core_laplacian_rbf(rbf)(x, c)
    Hfd = np.array([[(U.core_gradient_rbf(rbf)(x + e[j], c)[i] - U.core_gradient_rbf(rbf)(x - e[j], c)[i]) /
                     (2 * h) for j in range(2)] for i in range(2)])
    assert np.allclose(H, Hfd, rtol=1e-6, atol=1e-8) and H[0, 1] == H[1, 0]
    for mono in U.make_all_monomials(15):
        gm = U.core_gradient_mon(mono)(x)
        fd = np.array([(mono(x + e[i]) - mono(x - e[i])) / (2 * h) for i in range(2)])
        assert np.allclose(gm, fd, rtol=1e-6, atol=1e-9)
        Hm = U.core_laplacian_mon(mono)(x)
        Hmfd = np.array([[(U.core_gradient_mon(mono)(x + e[j])[i] - U.core_gradient_mon(mono)(x - e[j])[i]) /
                          (2 * h) for j in range(2)] for i in range(2)])
        assert np.allclose(Hm, Hmfd, rtol=1e-6, atol=1e-8)
