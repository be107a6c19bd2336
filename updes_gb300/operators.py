"""Drop-in ``pde_solver`` / ``pde_solver_jit`` and the nodal operators.

Mirrors the reference's public solve interface (updes/operators.py:15-111,
512-683): the same function names, argument meanings, facet/boundary
conventions and ``SteadySol(vals, coeffs, mat)`` result.  The work happens in
the CUDA library through the C ABI (``_lib``):

* the user's ``diff_operator`` is *captured*: it is called with probe values
  for ``nodal_value`` / ``nodal_gradient`` / ``nodal_laplacian`` /
  ``nodal_div_grad`` and must be linear in them; the result is a per-node
  weight table [value, d/dx, d/dy, d2/dx2, d2/dy2] that the assembly kernel
  applies with closed-form kernel derivatives;
* boundary conditions become row descriptors (Dirichlet, Neumann, Robin,
  periodic) in the reference's row order, with its quirks reproduced when
  ``compat_reference_quirks`` is on (the default);
* ``updes_solve`` assembles K = [[opΦ, opP], [bdΦ, bdP], [Pᵀ, 0]], factors it
  and refines in FP64; ``vals = [Φ P] c`` is evaluated on the GPU.
"""
from __future__ import annotations

import contextlib
import ctypes
import threading
from collections import namedtuple
from dataclasses import dataclass

import numpy as np

from . import _lib
from .rbf import rbf_spec

SteadySol = namedtuple("PDESolution", ["vals", "coeffs", "mat"])  # updes/utils.py:148


def compute_nb_monomials(max_degree, problem_dimension=2):
    """C(max_degree + dim, max_degree) (updes/utils.py:142-144)."""
    from math import comb
    return comb(max_degree + problem_dimension, max_degree)


# ---------------------------------------------------------------------------
# Solver options
# ---------------------------------------------------------------------------

@dataclass
class SolverOptions:
    precision: str = "fp32"            # "fp32": FP32 LU + FP64 GMRES refinement; "fp64": plain FP64 LU
    tol: float = 1e-13                 # relative residual of the equilibrated system
    max_iters: int = 200
    restart: int = 40
    fallback_fp64: bool = True         # refactor in FP64 when refinement stalls
    compat_reference_quirks: bool = True
    self_term: bool = False            # True: keep phi(0) on the diagonal of the Phi blocks
    reuse_factorization: bool = True   # reuse the last factors when the system (not the rhs) is unchanged

    def c_opts(self):
        o = _lib.SolveOpts()
        o.precision = {"fp64": _lib.PREC_FP64, "fp32": _lib.PREC_FP32}[self.precision]
        o.max_iters, o.restart = int(self.max_iters), int(self.restart)
        o.fallback_fp64, o.tol = int(bool(self.fallback_fp64)), float(self.tol)
        return o


DEFAULT_OPTIONS = SolverOptions()
LAST_INFO: dict = {}


# ---------------------------------------------------------------------------
# Nodal operators (updes/operators.py:15-111) with capture probes
# ---------------------------------------------------------------------------

_PROBE = threading.local()


@dataclass
class _Probe:
    value: float = 0.0
    gx: float = 0.0
    gy: float = 0.0
    lap: float = 0.0
    hxx: float = 0.0
    hyy: float = 0.0


class _Center:
    """Stand-in passed as ``center`` while capturing (not None, like a real center)."""

    def __repr__(self):
        return "<captured center>"


_CENTER = _Center()


def _monomial_terms(monomial, x):
    from .rbf import distance  # noqa: F401  (keeps module import order simple)
    px, py = _MONO_EXP[getattr(monomial, "keywords", {}).get("id", 0)] if hasattr(monomial, "keywords") else (0, 0)
    x0, x1 = float(x[0]), float(x[1])
    m = x0 ** px * x1 ** py
    mx = px * x0 ** (px - 1) * x1 ** py if px else 0.0
    my = py * x0 ** px * x1 ** (py - 1) if py else 0.0
    mxx = px * (px - 1) * x0 ** (px - 2) * x1 ** py if px > 1 else 0.0
    myy = py * (py - 1) * x0 ** px * x1 ** (py - 2) if py > 1 else 0.0
    return m, mx, my, mxx, myy


_MONO_EXP = [(0, 0), (1, 0), (0, 1), (2, 0), (1, 1), (0, 2), (3, 0), (2, 1), (1, 2), (0, 3), (4, 0), (3, 1),
             (2, 2), (1, 3), (0, 4)]


def make_monomial(x, id):
    """Monomial ``id`` at x (updes/utils.py:92-134)."""
    px, py = _MONO_EXP[id]
    return float(x[0]) ** px * float(x[1]) ** py


def make_all_monomials(nb_monomials):
    import functools
    return [functools.partial(make_monomial, id=j) for j in range(nb_monomials)]


def _rbf_terms_numeric(rbf, x, center):
    """(phi, gx, gy, hxx, hyy) of the kernel for one pair, closed form, NumPy."""
    from .rbf import KIND_NAMES
    kid, p = rbf_spec(rbf)
    s = np.asarray(x, dtype=np.float64) - np.asarray(center, dtype=np.float64)
    dx, dy = s
    r2 = dx * dx + dy * dy
    kind = KIND_NAMES[kid]
    if r2 == 0.0:
        return (0.0 if kind in ("polyharmonic", "thin_plate") else 1.0), 0.0, 0.0, 0.0, 0.0
    r = np.sqrt(r2)
    if kind == "polyharmonic":
        k = 2 * int(p) + 1
        phi, g1, g2 = r ** k, k * r ** (k - 2), k * (k - 2) * r ** (k - 4)
    elif kind == "gaussian":
        e2 = p * p
        phi = np.exp(-e2 * r2)
        g1, g2 = -2 * e2 * phi, 4 * e2 * e2 * phi
    elif kind == "multiquadric":
        e2 = p * p
        q = np.sqrt(1 + e2 * r2)
        phi, g1, g2 = q, e2 / q, -e2 * e2 / q ** 3
    elif kind == "inverse_multiquadric":
        e2 = p * p
        q = np.sqrt(1 + e2 * r2)
        phi, g1, g2 = 1 / q, -e2 / q ** 3, 3 * e2 * e2 / q ** 5
    else:
        a = int(p)
        lr = np.log(r)
        phi = lr * r ** (2 * a)
        g1 = r ** (2 * a - 2) * (2 * a * lr + 1)
        g2 = r ** (2 * a - 4) * (2 * a * (2 * a - 2) * lr + 4 * a - 2)
    return phi, g1 * dx, g1 * dy, g1 + g2 * dx * dx, g1 + g2 * dy * dy


def _rbf_hessian_offdiag(rbf, x, center):
    """d2/dxdy of the kernel for one pair (closed form, radial: g2 dx dy), 0 at r = 0."""
    from .rbf import KIND_NAMES
    kid, p = rbf_spec(rbf)
    dx, dy = np.asarray(x, dtype=np.float64) - np.asarray(center, dtype=np.float64)
    r2 = dx * dx + dy * dy
    if r2 == 0.0:
        return 0.0
    r = np.sqrt(r2)
    kind = KIND_NAMES[kid]
    if kind == "polyharmonic":
        k = 2 * int(p) + 1
        g2 = k * (k - 2) * r ** (k - 4)
    elif kind == "gaussian":
        g2 = 4 * p ** 4 * np.exp(-p * p * r2)
    elif kind == "multiquadric":
        g2 = -p ** 4 / np.sqrt(1 + p * p * r2) ** 3
    elif kind == "inverse_multiquadric":
        g2 = 3 * p ** 4 / np.sqrt(1 + p * p * r2) ** 5
    else:
        a = int(p)
        g2 = r ** (2 * a - 4) * (2 * a * (2 * a - 2) * np.log(r) + 4 * a - 2)
    return g2 * dx * dy


def core_gradient_rbf(rbf):
    """The kernel's gradient in x, as a function of (x, center) (updes/operators.py:34-35; closed form, 0
    where the reference's automatic derivative is NaN, at x = center)."""
    return lambda x, center: np.array(_rbf_terms_numeric(rbf, x, center)[1:3])


def core_gradient_mon(monomial):
    """The monomial's gradient, as a function of x (updes/operators.py:38-39)."""
    return lambda x: np.array(_monomial_terms(monomial, x)[1:3])


def core_laplacian_rbf(rbf):
    """The kernel's Hessian in x (2 x 2), as a function of (x, center): the reference's
    jacfwd(grad(rbf)), whose trace nodal_laplacian takes (updes/operators.py:63-65)."""
    def hess(x, center):
        t = _rbf_terms_numeric(rbf, x, center)
        h = _rbf_hessian_offdiag(rbf, x, center)
        return np.array([[t[3], h], [h, t[4]]])
    return hess


def core_laplacian_mon(monomial):
    """The monomial's Hessian (2 x 2), as a function of x (updes/operators.py:67-69)."""
    def hess(x):
        t = _monomial_terms(monomial, x)
        px, py = _MONO_EXP[getattr(monomial, "keywords", {}).get("id", 0)] if hasattr(monomial, "keywords") \
            else (0, 0)
        x0, x1 = float(x[0]), float(x[1])
        h = px * py * x0 ** (px - 1) * x1 ** (py - 1) if px and py else 0.0
        return np.array([[t[3], h], [h, t[4]]])
    return hess


def nodal_value(x, center=None, rbf=None, monomial=None):
    """RBF or monomial value at x (updes/operators.py:15-32)."""
    pr = getattr(_PROBE, "state", None)
    if pr is not None:
        return pr.value
    if center is not None:
        return _rbf_terms_numeric(rbf, x, center)[0]
    return _monomial_terms(monomial, x)[0]


def nodal_gradient(x, center=None, rbf=None, monomial=None):
    """Gradient w.r.t. x, 0 where undefined (updes/operators.py:42-60)."""
    pr = getattr(_PROBE, "state", None)
    if pr is not None:
        return np.array([pr.gx, pr.gy])
    t = _rbf_terms_numeric(rbf, x, center) if center is not None else _monomial_terms(monomial, x)
    return np.array([t[1], t[2]])


def nodal_laplacian(x, center=None, rbf=None, monomial=None):
    """Laplacian (trace of the Hessian) (updes/operators.py:70-85)."""
    pr = getattr(_PROBE, "state", None)
    if pr is not None:
        return pr.lap
    t = _rbf_terms_numeric(rbf, x, center) if center is not None else _monomial_terms(monomial, x)
    return t[3] + t[4]


def nodal_div_grad(x, center=None, rbf=None, monomial=None, args=None):
    """trace(W ⊙ H) with W built from ``args`` (updes/operators.py:88-111).

    Both of the reference's forms (array args -> rows [a0, a0], [a1, a1];
    tuple args -> rows [a0, a1], [a0, a1]) reduce to a0·H00 + a1·H11.
    """
    a0, a1 = args[0], args[1]
    pr = getattr(_PROBE, "state", None)
    if pr is not None:
        return a0 * pr.hxx + a1 * pr.hyy
    t = _rbf_terms_numeric(rbf, x, center) if center is not None else _monomial_terms(monomial, x)
    return a0 * t[3] + a1 * t[4]


@contextlib.contextmanager
def _probing(state):
    _PROBE.state = state
    try:
        yield
    finally:
        _PROBE.state = None


_BASIS = [dict(value=1.0), dict(gx=1.0), dict(gy=1.0), dict(lap=1.0), dict(hxx=1.0), dict(hyy=1.0)]
_STACKED_PROBE_MAX_NODES = 2048


def capture_operator(diff_operator, X, rbf, fields):
    """Per-node weights (m, 5) = [value, d/dx, d/dy, d2/dx2, d2/dy2] of a linear operator.

    ``X``: (m, 2) evaluation nodes; ``fields``: (F, m) per-node diff_args values.
    The operator is evaluated vectorised (x as (2, m), fields as (F, m)) when it
    accepts that, else node by node.  Raises ValueError if it is not a linear
    combination of the nodal operators.
    """
    m = X.shape[0]
    if fields is None:
        fields = np.ones((1, m))  # updes/assembly.py:114

    def run_vec(state):
        with _probing(state):
            out = diff_operator(X.T, _CENTER, rbf, None, fields)
        out = np.asarray(out, dtype=np.float64)
        if out.shape not in ((), (m,), (1,)):
            raise ValueError("shape")
        return np.broadcast_to(out, (m,)).copy()

    def run_loop(state):
        out = np.empty(m)
        with _probing(state):
            for i in range(m):
                out[i] = float(np.asarray(diff_operator(X[i], _CENTER, rbf, None, fields[:, i])))
        return out

    rng = np.random.default_rng(1234)
    rv = rng.uniform(0.5, 1.5, size=6)
    run = run_vec
    cols = None
    try:
        # All eight probes (zero, the six unit primitives, the random check) in one call: each primitive
        # returns a column of its eight probe values, which broadcasts against the (m,) node arrays into an
        # (8, m) result.  Kept only when its random-check row equals a separate evaluation of that probe.
        # It saves call overhead on small clouds; on large ones the (8, m) temporaries cost more than the
        # seven calls they replace (0.83 against 0.70 ms at m = 3,969), so those probe one by one.
        if m > _STACKED_PROBE_MAX_NODES:
            raise ValueError("large cloud")
        lanes = np.zeros((8, 6))
        lanes[1:7] = np.eye(6)
        lanes[7] = rv
        stacked = _Probe(*[lanes[:, k:k + 1] for k in range(6)])
        with _probing(stacked):
            out8 = np.asarray(diff_operator(X.T, _CENTER, rbf, None, fields), dtype=np.float64)
        out8 = np.broadcast_to(out8, (8, m)) if out8.shape in ((8, 1), (8, m)) else None
        if out8 is not None:
            check = run_vec(_Probe(*rv))
            if np.array_equal(check, out8[7]):
                base = out8[0].copy()
                cols = [out8[1 + k] - base for k in range(6)]
                got = check
    except Exception:
        cols = None
    if cols is None:
        try:
            base = run_vec(_Probe())
        except Exception:
            run = run_loop
            base = run_loop(_Probe())
        cols = [run(_Probe(**b)) - base for b in _BASIS]
        got = None
    if np.max(np.abs(base)) > 1e-12 * (1.0 + max(np.max(np.abs(c)) for c in cols)):
        raise ValueError("diff_operator has a term that does not multiply a nodal operator (it must be linear)")
    a, bx, by, lap, hxx, hyy = cols
    W = np.stack([a, bx, by, lap + hxx, lap + hyy], axis=-1)
    # linearity check on a random probe
    if got is None:
        got = run(_Probe(*rv))
    want = base + sum(c * v for c, v in zip(cols, rv))
    scale = 1.0 + np.max(np.abs(want))
    if np.max(np.abs(got - want)) > 1e-10 * scale:
        raise ValueError("diff_operator is not linear in nodal_value/nodal_gradient/nodal_laplacian/nodal_div_grad")
    return W


# ---------------------------------------------------------------------------
# Boundary conditions (updes/operators.py:512-555, 628-647)
# ---------------------------------------------------------------------------

def _eval_on_nodes(f, X):
    """Evaluate a callable of one point on the rows of X (vectorised when possible)."""
    m = X.shape[0]
    try:
        out = np.asarray(f(X.T), dtype=np.float64)
        if out.shape in ((), (m,), (1,)):
            return np.broadcast_to(out, (m,)).copy()
    except Exception:
        pass
    return np.array([float(np.asarray(f(X[i]))) for i in range(m)])


def boundary_conditions_func_to_arr(boundary_conditions, cloud):
    """Evaluate callable boundary conditions on their facet nodes (updes/operators.py:628-647)."""
    out = {}
    for f, bc in boundary_conditions.items():
        X = cloud.sorted_nodes[np.asarray(cloud.facet_nodes[f], dtype=np.int64)]
        if isinstance(bc, tuple):
            v, b = bc
            out[f] = (_eval_on_nodes(v, X) if callable(v) else v, _eval_on_nodes(b, X) if callable(b) else b)
        elif callable(bc):
            out[f] = _eval_on_nodes(bc, X)
        else:
            out[f] = bc
    return out


def _bc_values_and_betas(boundary_conditions, cloud, compat):
    """Facet values and per-node Robin coefficients (updes/operators.py:512-541)."""
    bcs = boundary_conditions_func_to_arr(boundary_conditions, cloud)
    q_vals = {}
    robin = {}
    for f, t in cloud.facet_types.items():
        if f not in bcs:
            raise AssertionError("facets and boundary functions don't match ids")  # assembly.py:474
        ids = cloud.facet_nodes[f]
        L = len(ids)
        bc = bcs[f]
        if t == "r":
            if isinstance(bc, tuple):
                vals, betas = bc
            else:
                vals, betas = bc, np.zeros(L)  # the reference warns and uses zeros
            betas = np.broadcast_to(np.asarray(betas, dtype=np.float64), (L,))
            for pos, i in enumerate(ids):
                ii = pos
                if compat:  # ii = i - node_ids[0] (operators.py:535), clamped to the array
                    ii = min(max(i - ids[0], 0), L - 1)
                robin[i] = float(betas[ii])
            bc = vals
        if t[0] == "p":
            q_vals[f] = np.zeros(L)  # zerofy_periodic_cond, operators.py:546-555
        else:
            q_vals[f] = np.broadcast_to(np.asarray(bc, dtype=np.float64), (L,)).copy()
    return q_vals, robin


def boundary_rows(cloud, robin, compat=True):
    """Row descriptors (kind, nodes (Nb,2), geom (Nb,8)) of the boundary rows, in the
    reference's order (updes/assembly.py:169-359)."""
    Ni, Nd, Nn, Nr = cloud.Ni, cloud.Nd, cloud.Nn, cloud.Nr
    N = cloud.N
    Nb = N - Ni
    son = cloud.sorted_outward_normals
    nrm = cloud.normals_by_node
    kind = np.zeros(Nb, np.int32)
    nodes = np.zeros((Nb, 2), np.int32)
    geom = np.zeros((Nb, 8))
    i = np.arange(Ni, Ni + Nd + Nn + Nr)
    r = i - Ni
    nodes[r, 0] = nodes[r, 1] = i
    kind[:Nd] = _lib.ROW_DIRICHLET
    sl_n = slice(Nd, Nd + Nn)
    kind[sl_n] = _lib.ROW_NEUMANN
    if Nn:
        geom[sl_n, 0:2] = son[np.arange(Nn)]
        geom[sl_n, 4:6] = nrm[Ni + Nd + np.arange(Nn)]
    sl_r = slice(Nd + Nn, Nd + Nn + Nr)
    kind[sl_r] = _lib.ROW_ROBIN
    if Nr:
        ir = Ni + Nd + Nn + np.arange(Nr)
        # bdΦ reads sorted_outward_normals[i - Ni - Nd - Nn] (assembly.py:206)
        geom[sl_r, 0:2] = son[ir - Ni - Nd - Nn] if compat else nrm[ir]
        geom[sl_r, 4:6] = nrm[ir]
        geom[sl_r, 6] = [robin.get(int(t), 0.0) for t in ir]
    half = sum(cloud.Np) // 2
    start, row = Ni + Nd + Nn + Nr, Nd + Nn + Nr
    for npts in cloud.Np:
        nc = npts // 2
        a = start + np.arange(nc)
        b = a + nc
        for rr, kd in ((row + np.arange(nc), _lib.ROW_PERIODIC_VALUE),
                       (row + half + np.arange(nc), _lib.ROW_PERIODIC_FLUX)):
            kind[rr] = kd
            nodes[rr, 0], nodes[rr, 1] = a, b
            geom[rr, 0:2] = son[a - Ni - Nd]
            geom[rr, 2:4] = son[b - Ni - Nd]
            geom[rr, 4:6] = nrm[a]
        row += nc
        start += npts
    return kind, nodes, geom


# ---------------------------------------------------------------------------
# Device side
# ---------------------------------------------------------------------------

def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("updes_gb300 needs a CUDA GPU (GB300); there is no CPU fallback")
    return torch


class DeviceProblem:
    """Device copies of one problem and the ``updes_problem`` struct pointing at them."""

    def __init__(self, cloud, rbf, max_degree, W, kind, bnodes, geom, self_term=False):
        torch = _torch()
        dev = torch.device("cuda", torch.cuda.current_device())
        self.torch = torch
        self.device = dev
        f64 = dict(dtype=torch.float64, device=dev)
        self.N, self.Ni = cloud.N, cloud.Ni
        self.M = compute_nb_monomials(max_degree)
        self.n = self.N + self.M
        self.kid, self.param = rbf_spec(rbf)
        self.nodes = torch.as_tensor(np.ascontiguousarray(cloud.sorted_nodes), **f64)
        self.W = torch.as_tensor(np.ascontiguousarray(W, dtype=np.float64).reshape(-1, 5), **f64)
        self.kind = torch.as_tensor(np.ascontiguousarray(kind, dtype=np.int32), device=dev)
        self.bnodes = torch.as_tensor(np.ascontiguousarray(bnodes, dtype=np.int32), device=dev)
        self.geom = torch.as_tensor(np.ascontiguousarray(geom, dtype=np.float64), **f64)
        sup = getattr(cloud, "sorted_local_supports", None)
        self.supports = None if sup is None else torch.as_tensor(np.ascontiguousarray(sup, dtype=np.int32),
                                                                 device=dev)
        p = _lib.Problem()
        p.N, p.Ni, p.M, p.rbf, p.rbf_param = self.N, self.Ni, self.M, self.kid, self.param
        p.self_term = int(bool(self_term))
        if self.supports is not None:
            p.support_width = int(self.supports.shape[1])
            p.supports = self.supports.data_ptr()
        p.nodes = self.nodes.data_ptr()
        p.op_weights = self.W.data_ptr() if self.Ni else None
        p.bd_kind = self.kind.data_ptr() if self.N > self.Ni else None
        p.bd_node = self.bnodes.data_ptr() if self.N > self.Ni else None
        p.bd_geom = self.geom.data_ptr() if self.N > self.Ni else None
        self.c = p

    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)


_WS_CACHE: dict = {}


def workspace(nbytes):
    """A cached device byte buffer of at least ``nbytes`` (reused between calls)."""
    torch = _torch()
    dev = torch.cuda.current_device()
    buf = _WS_CACHE.get(dev)
    if buf is None or buf.numel() < nbytes:
        _WS_CACHE.pop(dev, None)
        buf = torch.empty(int(nbytes), dtype=torch.uint8, device=torch.device("cuda", dev))
        _WS_CACHE[dev] = buf
    return buf


def free_workspace():
    _WS_CACHE.clear()


class _Factored:
    """A factorised system kept on the device: its problem arrays and workspace."""

    def __init__(self, key, dp, ws):
        self.key, self.dp, self.ws = key, dp, ws


_FACTOR_CACHE: dict = {}   # (device, slot) -> _Factored


def _system_key(cloud, rbf, max_degree, W, kind, bnodes, geom, opts):
    import hashlib
    h = hashlib.sha1()
    sup = getattr(cloud, "sorted_local_supports", None)
    for a in (np.ascontiguousarray(cloud.sorted_nodes), np.ascontiguousarray(W), np.ascontiguousarray(kind),
              np.ascontiguousarray(bnodes), np.ascontiguousarray(geom),
              np.zeros(0, np.int32) if sup is None else np.ascontiguousarray(sup)):
        h.update(a.tobytes())
    return (rbf_spec(rbf), int(max_degree), opts.precision, bool(opts.self_term), h.hexdigest())


def solve_device(dp: DeviceProblem, q, opts: SolverOptions, want_vals=True, key=None, slot="main"):
    """Solve on device tensors; returns (coeffs, vals, info dict).

    With ``key`` (a description of the system) the factorisation is cached per
    device and ``slot``: a later call with the same key solves against the
    stored factors (``updes_solve_factored``) instead of refactoring.
    Without it every call is a fresh ``updes_solve``.
    """
    torch = dp.torch
    lib = _lib.load()
    q = torch.as_tensor(q, dtype=torch.float64, device=dp.device).contiguous()
    coeffs = torch.empty(dp.n, dtype=torch.float64, device=dp.device)
    vals = torch.empty(dp.N, dtype=torch.float64, device=dp.device) if want_vals else None
    co = opts.c_opts()
    nbytes = ctypes.c_size_t()
    _lib.check(lib.updes_solve_workspace(ctypes.byref(dp.c), ctypes.byref(co), ctypes.byref(nbytes)),
               "updes_solve_workspace")
    info = _lib.SolveInfo()
    if key is None:
        ws = workspace(nbytes.value)
        st = lib.updes_solve(ctypes.byref(dp.c), q.data_ptr(), coeffs.data_ptr(),
                             vals.data_ptr() if vals is not None else None, ctypes.byref(co), ctypes.byref(info),
                             ws.data_ptr(), ws.numel(), dp.stream())
        what = "updes_solve"
    else:
        ck = (dp.device.index, slot)
        ent = _FACTOR_CACHE.get(ck)
        if ent is None or ent.key != key:
            old = ent.ws if ent is not None and ent.ws.numel() >= nbytes.value else None
            _FACTOR_CACHE.pop(ck, None)
            ws = old if old is not None else torch.empty(nbytes.value, dtype=torch.uint8, device=dp.device)
            fi = _lib.SolveInfo()
            st = lib.updes_factor(ctypes.byref(dp.c), ctypes.byref(co), ctypes.byref(fi), ws.data_ptr(), ws.numel(),
                                  dp.stream())
            _lib.check(st, "updes_factor")
            ent = _Factored(key, dp, ws)
            _FACTOR_CACHE[ck] = ent
        else:
            fi = None
        st = lib.updes_solve_factored(ctypes.byref(ent.dp.c), 1, q.data_ptr(), 1, coeffs.data_ptr(), 1,
                                      vals.data_ptr() if vals is not None else None, 1, ctypes.byref(co),
                                      ctypes.byref(info), ent.ws.data_ptr(), ent.ws.numel(), dp.stream())
        if fi is not None:
            info.t_assemble_ms, info.t_factor_ms = fi.t_assemble_ms, fi.t_factor_ms + info.t_factor_ms
            info.lu_info = fi.lu_info
        what = "updes_solve_factored"
    d = info.as_dict()
    d["reused_factors"] = key is not None and fi is None
    LAST_INFO.clear()
    LAST_INFO.update(d)
    _lib.check(st, what)
    return coeffs, vals, d


def free_factorizations():
    _FACTOR_CACHE.clear()


def eval_field(points, coeffs, centers, rbf, what=0):
    """value (0) / gradient (1) / laplacian (2) of a field at points (m, 2), on the GPU."""
    torch = _torch()
    lib = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    P = torch.as_tensor(np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 2), device=dev)
    C = torch.as_tensor(np.ascontiguousarray(centers, dtype=np.float64).reshape(-1, 2), device=dev)
    c = torch.as_tensor(np.ascontiguousarray(coeffs, dtype=np.float64), device=dev)
    m, N = P.shape[0], C.shape[0]
    M = c.shape[0] - N
    out = torch.empty((m, 2) if what == 1 else (m,), dtype=torch.float64, device=dev)
    kid, param = rbf_spec(rbf)
    st = lib.updes_eval_field(m, P.data_ptr(), N, C.data_ptr(), M, kid, param, c.data_ptr(), what,
                              out.data_ptr(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "updes_eval_field")
    return out.cpu().numpy()


# ---------------------------------------------------------------------------
# Field operators (updes/operators.py:118-371) and coefficients (assembly.py:404-430)
# ---------------------------------------------------------------------------

def _points(x):
    x = np.asarray(x, dtype=np.float64)
    if x.ndim == 1:
        return x[None, :], True
    if x.ndim == 2 and x.shape[0] == 2 and x.shape[1] != 2:
        return x.T, False        # (2, m): a vectorised call from pde_solver
    return x, False


def value(x, field, centers, rbf=None, clip_val=None):
    """Field value from coefficients (updes/operators.py:118-147)."""
    P, single = _points(x)
    out = eval_field(P, field, centers, rbf, 0)
    if clip_val:
        out = np.clip(out, -clip_val, clip_val)
    return out[0] if single else out


def gradient(x, field, centers, rbf=None, clip_val=None):
    """Field gradient from coefficients (updes/operators.py:156-184)."""
    P, single = _points(x)
    out = eval_field(P, field, centers, rbf, 1)
    if clip_val:
        out = np.clip(out, -clip_val, clip_val)
    return out[0] if single else out


def laplacian(x, field, centers, rbf=None, clip_val=None):
    """Field Laplacian from coefficients (updes/operators.py:319-348)."""
    P, single = _points(x)
    out = eval_field(P, field, centers, rbf, 2)
    if clip_val:
        out = np.clip(out, -clip_val, clip_val)
    return out[0] if single else out


def value_vec(xs, field, centers, rbf=None):
    return value(np.asarray(xs).reshape(-1, 2), field, centers, rbf)


def gradient_vec(xs, field, centers, rbf=None):
    return gradient(np.asarray(xs).reshape(-1, 2), field, centers, rbf)


def laplacian_vec(xs, field, centers, rbf=None):
    return laplacian(np.asarray(xs).reshape(-1, 2), field, centers, rbf)


def divergence(x, field, centers, rbf=None, clip_val=None):
    """d/dx of field[..., 0] + d/dy of field[..., 1] (updes/operators.py:294-312)."""
    field = np.asarray(field)
    gx = gradient(x, field[..., 0], centers, rbf)
    gy = gradient(x, field[..., 1], centers, rbf)
    out = np.asarray(gx)[..., 0] + np.asarray(gy)[..., 1]
    return np.clip(out, -clip_val, clip_val) if clip_val else out


def _interp_problem(cloud, rbf, max_degree):
    """The interpolation system A = [[Φ, P], [Pᵀ, 0]]: every row a value row."""
    Nb = cloud.N
    kind = np.full(Nb, _lib.ROW_DIRICHLET, np.int32)
    nodes = np.repeat(np.arange(Nb, dtype=np.int32)[:, None], 2, axis=1)
    geom = np.zeros((Nb, 8))

    class _C:
        pass
    c = _C()
    c.N, c.Ni, c.sorted_nodes = cloud.N, 0, cloud.sorted_nodes
    c.sorted_local_supports = getattr(cloud, "sorted_local_supports", None)  # A's Phi keeps the same supports
    return DeviceProblem(c, rbf, max_degree, np.zeros((0, 5)), kind, nodes, geom)


def core_compute_coefficients(field, cloud, rbf, nb_monomials, options=None):
    """c = A^-1 [field; 0] (updes/assembly.py:404-410), solved on the GPU."""
    deg = {1: 0, 3: 1, 6: 2, 10: 3, 15: 4}[nb_monomials]
    dp = _interp_problem(cloud, rbf, deg)
    o = options or SolverOptions(precision="fp64")
    key = None
    if o.reuse_factorization:
        key = ("interp",) + _system_key(cloud, rbf, deg, np.zeros((0, 5)), np.zeros(0, np.int32),
                                        np.zeros((0, 2), np.int32), np.zeros((0, 8)), o)
    coeffs, _, _ = solve_device(dp, np.asarray(field, dtype=np.float64), o, want_vals=False, key=key, slot="interp")
    return coeffs.cpu().numpy()


def compute_coefficients(field, cloud, rbf, max_degree, options=None):
    """updes/assembly.py:413-418."""
    return core_compute_coefficients(field, cloud, rbf, compute_nb_monomials(max_degree), options)


get_field_coefficients = compute_coefficients  # updes/assembly.py:423-430


# ---------------------------------------------------------------------------
# The solver (updes/operators.py:559-683)
# ---------------------------------------------------------------------------

class CollocationMatrix:
    """The reference's ``SteadySol.mat`` = B = [opΦ opP; bdΦ bdP] · inv(A)[:, :N].

    B is never formed on the hot path (the solve factors the Kansa matrix
    instead); ``materialize()`` builds it on demand with O(n³) work.
    """

    def __init__(self, build):
        self._build = build
        self._B = None

    def materialize(self):
        if self._B is None:
            self._B = self._build()
        return self._B

    def __array__(self, dtype=None, copy=None):
        B = self.materialize()
        return B.astype(dtype) if dtype is not None else B

    @property
    def shape(self):
        return self.materialize().shape


def prepare(diff_operator, rhs_operator, cloud, boundary_conditions, rbf, max_degree, diff_args=None,
            rhs_args=None, options=None):
    """Host-side preparation: operator capture, row descriptors and q (no GPU solve yet)."""
    opts = options or DEFAULT_OPTIONS
    N, Ni = cloud.N, cloud.Ni
    X = cloud.sorted_nodes
    M = compute_nb_monomials(max_degree)
    _require_finite(X, "the cloud's node coordinates")
    _require_distinct(X)
    fields = None
    if diff_args:
        fields = np.stack([np.asarray(a, dtype=np.float64) for a in diff_args])  # (F, N)
        _require_finite(fields, "diff_args")
    W = capture_operator(diff_operator, X[:Ni], rbf, None if fields is None else fields[:, :Ni]) if Ni else \
        np.zeros((0, 5))
    _require_finite(W, "the captured operator weights")
    q_vals, robin = _bc_values_and_betas(boundary_conditions, cloud, opts.compat_reference_quirks)
    kind, bnodes, geom = boundary_rows(cloud, robin, opts.compat_reference_quirks)
    # rhs (updes/assembly.py:434-485)
    q = np.zeros(N)
    if Ni:
        fc = None
        if rhs_args is not None:
            cols = []
            for fld in rhs_args:
                fld = np.asarray(fld, dtype=np.float64)
                cols.append(core_compute_coefficients(fld, cloud, rbf, M) if fld.shape[0] == N else fld)
            fc = np.stack(cols, axis=-1)
        Xi = X[:Ni]
        try:
            out = np.asarray(rhs_operator(Xi.T, X, rbf, fc), dtype=np.float64)
            if out.shape not in ((), (Ni,), (1,)):
                raise ValueError("shape")
            q[:Ni] = np.broadcast_to(out, (Ni,))
        except Exception:
            q[:Ni] = [float(np.asarray(rhs_operator(Xi[i], X, rbf, fc))) for i in range(Ni)]
    for f, v in q_vals.items():
        q[np.asarray(cloud.facet_nodes[f], dtype=np.int64)] = v
    _require_finite(q, "the right-hand side (rhs_operator and boundary values)")
    _require_finite(geom, "the Robin coefficients")
    return W, kind, bnodes, geom, q


def _require_distinct(X):
    """Two nodes at the same place make two identical rows of the collocation matrix: it is singular, and an
    LU then meets a pivot at rounding level rather than an exact zero (LAPACK's too), so the solve would
    return noise.  Rejected on the host (the reference solves it silently)."""
    # each node as one complex number x + iy: NumPy sorts complex values by real, then imaginary part
    Z = np.ascontiguousarray(X, dtype=np.float64).view(np.complex128).ravel()
    order = np.argsort(Z, kind="stable")
    same = Z[order[1:]] == Z[order[:-1]]
    if np.any(same):
        k = int(np.flatnonzero(same)[0])
        i, j = sorted((int(order[k]), int(order[k + 1])))
        at = tuple(float(v) for v in X[i])
        raise ValueError(f"nodes {i} and {j} (sorted order) coincide at {at}: the collocation matrix would be singular")


def _require_finite(a, what):
    """NaN or inf in a problem's data is rejected before any GPU work (the reference would return NaN)."""
    a = np.asarray(a)
    if a.size and not np.all(np.isfinite(a)):
        bad = int(np.size(a) - np.count_nonzero(np.isfinite(a)))
        raise ValueError(f"{what}: {bad} entries are not finite (NaN or inf)")


def pde_solver(diff_operator, rhs_operator, cloud, boundary_conditions, rbf, max_degree, diff_args=None,
               rhs_args=None, options=None):
    """Solve a linear PDE by global RBF collocation on the GPU (updes/operators.py:559-618).

    Returns ``SteadySol(vals, coeffs, mat)`` with ``vals`` (N,) in
    ``cloud.sorted_nodes`` order, ``coeffs`` (N + M,) and ``mat`` a lazy
    ``CollocationMatrix`` (the reference's B).
    """
    opts = options or DEFAULT_OPTIONS
    W, kind, bnodes, geom, q = prepare(diff_operator, rhs_operator, cloud, boundary_conditions, rbf, max_degree,
                                       diff_args, rhs_args, opts)
    dp = DeviceProblem(cloud, rbf, max_degree, W, kind, bnodes, geom, opts.self_term)
    key = _system_key(cloud, rbf, max_degree, W, kind, bnodes, geom, opts) if opts.reuse_factorization else None
    coeffs, vals, _ = solve_device(dp, q, opts, key=key)
    coeffs_h = coeffs.cpu().numpy()
    vals_h = vals.cpu().numpy()

    def build_B():
        return materialize_B(dp, cloud, rbf, max_degree)
    return SteadySol(vals_h, coeffs_h, CollocationMatrix(build_B))


def pde_solver_jit(diff_operator, rhs_operator, cloud, boundary_conditions, rbf, max_degree, diff_args=None,
                   rhs_args=None, options=None):
    """Same as ``pde_solver`` after evaluating callable BCs (updes/operators.py:650-683)."""
    bcs = boundary_conditions_func_to_arr(boundary_conditions, cloud)
    return pde_solver(diff_operator, rhs_operator, cloud, bcs, rbf, max_degree, diff_args, rhs_args, options)


pde_solver_jit_with_bc = pde_solver


def pde_multi_solver(diff_operators, rhs_operators, cloud, boundary_conditions, rbf, max_degree, nb_iters=10,
                     tol=1e-6, diff_args=None, rhs_args=None, options=None):
    """Solve a system of (non-linear) PDEs by Picard sweeps (updes/operators.py:686-771).

    ``diff_operators``, ``rhs_operators`` and ``boundary_conditions`` hold one entry per scalar field.
    Each of ``nb_iters`` sweeps solves every field's PDE with ``pde_solver``; the first ``n`` diff_args
    of every PDE are the previous sweep's values of the ``n`` fields (initially ``diff_args[0][:n]``) and
    the rest of ``diff_args[i]`` and all of ``rhs_args[i]`` stay fixed.  All fields of a sweep see the
    same previous values (Jacobi order), and the last sweep's ``SteadySol`` list is returned.  As in the
    reference, ``tol`` does not stop the sweeps early; the relative change of each sweep (the quantity
    the reference computes) is left in ``LAST_MULTI_INFO["changes"]``.  Fields whose operator weights do
    not change between solves reuse their factorisation (``SolverOptions.reuse_factorization``).
    """
    n = len(diff_operators)
    if not (n == len(rhs_operators) == len(boundary_conditions)):
        raise AssertionError("The number of differential operators must match the number of right-hand side "
                             "operators")
    if diff_args is None or len(diff_args) < 1 or len(diff_args[0]) < n:
        raise ValueError("diff_args[0] must start with the initial values of the fields")
    rhs_args = rhs_args if rhs_args is not None else [None] * n
    bcs = [boundary_conditions_func_to_arr(b, cloud) for b in boundary_conditions]
    host = lambda u: u.detach().cpu().numpy() if hasattr(u, "detach") else u
    vals = [np.asarray(host(u), dtype=np.float64) for u in diff_args[0][:n]]
    changes = []
    sols = []
    for _ in range(int(nb_iters)):
        sols = [pde_solver(diff_operators[i], rhs_operators[i], cloud, bcs[i], rbf, max_degree,
                           diff_args=list(vals) + list(diff_args[i][n:]), rhs_args=rhs_args[i], options=options)
                for i in range(n)]
        changes.append(float(sum(np.linalg.norm(sols[i].vals - vals[i]) / (np.linalg.norm(vals[i]) + 1e-14)
                                 for i in range(n))))
        vals = [s.vals for s in sols]
    LAST_MULTI_INFO.clear()
    LAST_MULTI_INFO.update(changes=changes, tol=tol)
    return sols


LAST_MULTI_INFO: dict = {}


def materialize_B(dp, cloud, rbf, max_degree):
    """B = K[:N] · inv(A)[:, :N] in FP64 on the GPU (O(n³); diagnostics only)."""
    torch = dp.torch
    lib = _lib.load()
    n, N = dp.n, dp.N
    ld = int(lib.updes_matrix_ld(n, 8))
    K = torch.zeros((n, ld), dtype=torch.float64, device=dp.device)
    _lib.check(lib.updes_assemble(ctypes.byref(dp.c), K.data_ptr(), ld, None, 0, dp.stream()), "updes_assemble")
    ap = _interp_problem(cloud, rbf, max_degree)
    A = torch.zeros((n, ld), dtype=torch.float64, device=dp.device)
    _lib.check(lib.updes_assemble(ctypes.byref(ap.c), A.data_ptr(), ld, None, 0, dp.stream()), "updes_assemble")
    # B^T = inv(A)^T[:N, :] K[:N]^T  ->  solve A^T Y = K[:N]^T, B = Y^T[:, :N]
    Y = K[:N, :n].T.contiguous()  # (n, N)
    piv = torch.empty(2 * n, dtype=torch.int32, device=dp.device)
    nbytes = ctypes.c_size_t()
    _lib.check(lib.updes_lu_workspace(n, _lib.PREC_FP64, ctypes.byref(nbytes)), "updes_lu_workspace")
    ws = torch.empty(nbytes.value + 8 * n + 512, dtype=torch.uint8, device=dp.device)
    info = ctypes.c_int32()
    _lib.check(lib.updes_lu_factor(n, A.data_ptr(), ld, _lib.PREC_FP64, None, 0, piv.data_ptr(), ws.data_ptr(),
                                   ws.numel(), ctypes.byref(info), dp.stream()), "updes_lu_factor")
    _lib.check(lib.updes_lu_solve(n, A.data_ptr(), ld, _lib.PREC_FP64, piv.data_ptr(), Y.data_ptr(), N, N, 1,
                                  ws.data_ptr(), ws.numel(), dp.stream()), "updes_lu_solve")
    return Y.T[:, :N].cpu().numpy().copy()


def pde_solver_many(systems, options=None, streams=8):
    """Solve many independent systems in one call (``updes_solve_many``).

    ``systems``: a sequence of dicts with the keyword arguments of ``pde_solver``
    (``diff_operator``, ``rhs_operator``, ``cloud``, ``boundary_conditions``,
    ``rbf``, ``max_degree`` and optionally ``diff_args``, ``rhs_args``); callable
    boundary conditions are evaluated as in ``pde_solver_jit``.  Returns a list of
    ``SteadySol`` in the same order.  The solves run on ``streams`` CUDA streams
    at once, largest system first; each is exactly ``pde_solver``'s solve.
    """
    torch = _torch()
    lib = _lib.load()
    opts = options or DEFAULT_OPTIONS
    dps, qs = [], []
    for sysd in systems:
        cloud = sysd["cloud"]
        bcs = boundary_conditions_func_to_arr(sysd["boundary_conditions"], cloud)
        W, kind, bnodes, geom, q = prepare(sysd["diff_operator"], sysd["rhs_operator"], cloud, bcs, sysd["rbf"],
                                           sysd["max_degree"], sysd.get("diff_args"), sysd.get("rhs_args"), opts)
        dp = DeviceProblem(cloud, sysd["rbf"], sysd["max_degree"], W, kind, bnodes, geom, opts.self_term)
        dps.append(dp)
        qs.append(torch.as_tensor(q, dtype=torch.float64, device=dp.device))
    count = len(dps)
    if count == 0:
        return []
    coeffs = [torch.empty(dp.n, dtype=torch.float64, device=dp.device) for dp in dps]
    vals = [torch.empty(dp.N, dtype=torch.float64, device=dp.device) for dp in dps]
    probs = (_lib.Problem * count)(*[dp.c for dp in dps])
    ptrs = lambda ts: (ctypes.c_void_p * count)(*[t.data_ptr() for t in ts])
    qp, cp, vp = ptrs(qs), ptrs(coeffs), ptrs(vals)
    infos = (_lib.SolveInfo * count)()
    co = opts.c_opts()
    nbytes = ctypes.c_size_t()
    _lib.check(lib.updes_solve_many_workspace(probs, count, ctypes.byref(co), int(streams), ctypes.byref(nbytes)),
               "updes_solve_many_workspace")
    ws = torch.empty(nbytes.value, dtype=torch.uint8, device=dps[0].device)
    torch.cuda.synchronize()  # the library's streams do not order with the caller's
    st = lib.updes_solve_many(probs, count, ctypes.cast(qp, ctypes.c_void_p), ctypes.cast(cp, ctypes.c_void_p),
                              ctypes.cast(vp, ctypes.c_void_p), ctypes.byref(co), infos, ws.data_ptr(), ws.numel(),
                              int(streams))
    LAST_MANY_INFO[:] = [infos[i].as_dict() for i in range(count)]
    _lib.check(st, "updes_solve_many")
    out = []
    for sysd, dp, c, v in zip(systems, dps, coeffs, vals):
        cloud, rbf, deg = sysd["cloud"], sysd["rbf"], sysd["max_degree"]
        out.append(SteadySol(v.cpu().numpy(), c.cpu().numpy(),
                             CollocationMatrix(lambda dp=dp, cloud=cloud, rbf=rbf, deg=deg:
                                               materialize_B(dp, cloud, rbf, deg))))
    return out


LAST_MANY_INFO: list = []
