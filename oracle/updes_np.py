"""FP64 NumPy/SciPy restatement of Updes' global RBF collocation path.

TEST INFRASTRUCTURE — this module is the oracle.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it, and only as the checker.  The product
(``updes_gb300``) never imports it.

Parity pin: every function here is checked against golden vectors produced by
running the reference package itself (``updes`` 1.0.3, imported unmodified
with a torch-backed stand-in for jax, ``tests/golden/make_golden.py``).

Reference citations are ``path:line`` inside the Updes source tree.

Contents
--------
* ``square_cloud``      — ``updes/cloud.py:382-510`` (SquareCloud), ``:115-172`` (renumber_nodes)
* ``rbf_terms``         — ``updes/utils.py:19-69`` (kernels) and the AD derivatives of
                          ``updes/operators.py:15-111`` restated in closed form
* ``monomial_terms``    — ``updes/utils.py:92-144``
* ``boundary_rows``     — row descriptors for ``updes/assembly.py:141-362``
* ``assemble_K``        — the augmented Kansa matrix [[opΦ, opP], [bdΦ, bdP], [Pᵀ, 0]]
* ``assemble_A``        — ``updes/assembly.py:10-85``
* ``solve_faithful``    — ``updes/operators.py:559-618`` (inv → GEMM → QR → inv)
* ``solve_direct``      — LU of the Kansa matrix (same solution, one factorisation)
* ``value`` / ``gradient`` — ``updes/operators.py:118-184``
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla

# ---------------------------------------------------------------------------
# RBF kernels and their closed-form derivatives
# ---------------------------------------------------------------------------

RBF_KINDS = ("polyharmonic", "gaussian", "multiquadric", "inverse_multiquadric", "thin_plate")

# Monomial exponents by id: updes/utils.py:103-132 (ids 0..14).
MONOMIAL_EXPONENTS = [(0, 0), (1, 0), (0, 1), (2, 0), (1, 1), (0, 2), (3, 0), (2, 1), (1, 2),
                      (0, 3), (4, 0), (3, 1), (2, 2), (1, 3), (0, 4)]


def nb_monomials(max_degree: int, dim: int = 2) -> int:
    """updes/utils.py:142-144: C(max_degree + dim, max_degree)."""
    return math.comb(max_degree + dim, max_degree)


def rbf_terms(kind: str, param: float, dx, dy):
    """Kernel value, gradient (w.r.t. the evaluation point) and Hessian diagonal.

    ``dx, dy`` = x − center.  Returns ``(phi, gx, gy, hxx, hyy)``.

    Value: updes/utils.py:30-69.  Derivatives: the reference differentiates the
    kernel with jax.grad / jax.jacfwd(jax.grad) (updes/operators.py:34-85) and
    then applies ``nan_to_num``; at r = 0 every derivative is 0/0 → NaN → 0, so
    the derivatives are 0 there.  For r > 0 the closed forms below are exact:
    with f = f(r), g1 = f'/r, g2 = (f'' − f'/r)/r²:
    ∇ = g1·s, ∂xx = g1 + g2·dx², ∂yy = g1 + g2·dy².
    """
    dx = np.asarray(dx, dtype=np.float64)
    dy = np.asarray(dy, dtype=np.float64)
    r2 = dx * dx + dy * dy
    r = np.sqrt(r2)
    zero = r2 == 0.0
    rs = np.where(zero, 1.0, r)          # safe r for the r>0 branch
    with np.errstate(all="ignore"):
        if kind == "polyharmonic":
            k = 2 * int(param) + 1                 # r^(2a+1), updes/utils.py:50-51
            phi = rs ** k
            g1 = k * rs ** (k - 2)
            g2 = k * (k - 2) * rs ** (k - 4)
            phi0 = 0.0
        elif kind == "gaussian":
            e2 = param * param                     # exp(-(eps r)^2), updes/utils.py:44-45
            phi = np.exp(-e2 * rs * rs)
            g1 = -2.0 * e2 * phi
            g2 = 4.0 * e2 * e2 * phi
            phi0 = 1.0
        elif kind == "multiquadric":
            e2 = param * param                     # sqrt(1+(eps r)^2), updes/utils.py:30-31
            q = np.sqrt(1.0 + e2 * rs * rs)
            phi = q
            g1 = e2 / q
            g2 = -e2 * e2 / (q * q * q)
            phi0 = 1.0
        elif kind == "inverse_multiquadric":
            e2 = param * param                     # 1/sqrt(1+(eps r)^2), updes/utils.py:37-38
            q = np.sqrt(1.0 + e2 * rs * rs)
            phi = 1.0 / q
            g1 = -e2 / (q * q * q)
            g2 = 3.0 * e2 * e2 / (q ** 5)
            phi0 = 1.0
        elif kind == "thin_plate":
            a = int(param)                         # nan_to_num(log r · r^(2a)), updes/utils.py:63-65
            lr = np.log(rs)
            phi = lr * rs ** (2 * a)
            g1 = rs ** (2 * a - 2) * (2 * a * lr + 1.0)
            g2 = rs ** (2 * a - 4) * (2 * a * (2 * a - 2) * lr + 4 * a - 2)
            phi0 = 0.0
        else:
            raise ValueError(f"unknown rbf kind {kind!r}")
        gx = g1 * dx
        gy = g1 * dy
        hxx = g1 + g2 * dx * dx
        hyy = g1 + g2 * dy * dy
    phi = np.where(zero, phi0, phi)
    gx = np.where(zero, 0.0, gx)
    gy = np.where(zero, 0.0, gy)
    hxx = np.where(zero, 0.0, hxx)
    hyy = np.where(zero, 0.0, hyy)
    return phi, gx, gy, hxx, hyy


def monomial_terms(k: int, x, y):
    """Value, gradient and Hessian diagonal of monomial ``k`` (updes/utils.py:92-134)."""
    px, py = MONOMIAL_EXPONENTS[k]
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)

    def pw(b, e):
        return np.ones_like(b) if e == 0 else b ** e

    m = pw(x, px) * pw(y, py)
    mx = px * pw(x, px - 1) * pw(y, py) if px > 0 else np.zeros_like(x)
    my = py * pw(x, px) * pw(y, py - 1) if py > 0 else np.zeros_like(x)
    mxx = px * (px - 1) * pw(x, px - 2) * pw(y, py) if px > 1 else np.zeros_like(x)
    myy = py * (py - 1) * pw(x, px) * pw(y, py - 2) if py > 1 else np.zeros_like(x)
    return m, mx, my, mxx, myy


# ---------------------------------------------------------------------------
# SquareCloud restatement (updes/cloud.py:382-510, 115-172)
# ---------------------------------------------------------------------------

@dataclass
class Cloud:
    Nx: int
    Ny: int
    facet_types: dict            # facet -> "d" | "n" | "r" | "p<tag><index>" (as stored by Cloud.__init__)
    N: int = 0
    Ni: int = 0
    Nd: int = 0
    Nn: int = 0
    Nr: int = 0
    Np: list = field(default_factory=list)
    sorted_nodes: np.ndarray = None          # (N, 2) in renumbered order
    node_types: dict = None                  # renumbered id -> type string
    facet_nodes: dict = None                 # facet -> renumbered ids (original-id order)
    outward_normals: dict = None             # renumbered id -> (2,)
    sorted_outward_normals: np.ndarray = None
    renumbering_map: dict = None             # original id -> renumbered id
    dim: int = 2


def square_cloud(Nx: int, Ny: int, facet_types: dict, coords=None) -> Cloud:
    """Build a SquareCloud exactly as updes/cloud.py:382-408 orders it.

    ``coords``: optional (Nx*Ny, 2) node coordinates indexed by ORIGINAL global
    id (id = i*Ny + j, updes/cloud.py:411-422); defaults to the uniform grid of
    updes/cloud.py:427-446 (node (i, j) at (x_i, y_j)).
    """
    # Cloud.__init__ appends the facet's position to periodic types (updes/cloud.py:42-49).
    ft = {}
    for idx, (k, v) in enumerate(facet_types.items()):
        ft[k] = v + str(idx) if v[0] == "p" else v
    N = Nx * Ny
    rev = {}
    for i in range(Nx):
        for j in range(Ny):
            rev[i * Ny + j] = (i, j)
    # define_node_types: corner precedence North > South > East > West (cloud.py:455-470)
    facet_nodes = {k: [] for k in ft}
    node_types = {}
    for g in range(N):
        i, j = rev[g]
        if j == Ny - 1:
            facet_nodes["North"].append(g); node_types[g] = ft["North"]
        elif j == 0:
            facet_nodes["South"].append(g); node_types[g] = ft["South"]
        elif i == Nx - 1:
            facet_nodes["East"].append(g); node_types[g] = ft["East"]
        elif i == 0:
            facet_nodes["West"].append(g); node_types[g] = ft["West"]
        else:
            node_types[g] = "i"
    Nd = sum(len(facet_nodes[f]) for f, t in ft.items() if t == "d")
    Nn = sum(len(facet_nodes[f]) for f, t in ft.items() if t == "n")
    Nr = sum(len(facet_nodes[f]) for f, t in ft.items() if t == "r")
    npd = {}
    for f, t in ft.items():
        if t[0] == "p":
            npd[t[:-1]] = npd.get(t[:-1], 0) + len(facet_nodes[f])
    Np = [npd[k] for k in sorted(npd)]
    Ni = N - Nd - Nn - Nr - sum(Np)
    # coordinates (cloud.py:425-446)
    if coords is None:
        xs = np.linspace(0.0, 1.0, Nx)
        ys = np.linspace(0.0, 1.0, Ny)
        coords = np.array([[xs[rev[g][0]], ys[rev[g][1]]] for g in range(N)])
    coords = np.asarray(coords, dtype=np.float64)
    # outward normals for n, r, p nodes (cloud.py:493-510)
    normals = {}
    for g in range(N):
        if node_types[g][0] in ("n", "r", "p"):
            i, j = rev[g]
            if j == Ny - 1:
                nv = (0.0, 1.0)
            elif j == 0:
                nv = (0.0, -1.0)
            elif i == Nx - 1:
                nv = (1.0, 0.0)
            else:
                nv = (-1.0, 0.0)
            normals[g] = np.array(nv)
    # renumbering: internal, dirichlet, neumann, robin, periodic (cloud.py:124-150)
    lists = {"i": [], "d": [], "n": [], "r": []}
    pn = {}
    for g in range(N):
        t = node_types[g]
        if t[0] == "p":
            pn.setdefault(t, []).append(g)
        else:
            lists[t[0]].append(g)
    allp = []
    for k in sorted(pn):
        allp += pn[k]
    order = lists["i"] + lists["d"] + lists["n"] + lists["r"] + allp
    new = {v: k for k, v in enumerate(order)}
    c = Cloud(Nx=Nx, Ny=Ny, facet_types=ft, N=N, Ni=Ni, Nd=Nd, Nn=Nn, Nr=Nr, Np=Np)
    c.sorted_nodes = coords[order].copy()
    c.node_types = {new[g]: node_types[g] for g in range(N)}
    c.facet_nodes = {f: [new[g] for g in ids] for f, ids in facet_nodes.items()}
    c.outward_normals = {new[g]: v for g, v in normals.items()}
    keys = sorted(c.outward_normals)
    c.sorted_outward_normals = (np.stack([c.outward_normals[k] for k in keys])
                                if keys else np.zeros((0, 2)))
    c.renumbering_map = new
    return c


def local_supports(sorted_nodes: np.ndarray, support_size: int) -> np.ndarray:
    """Local supports (updes/cloud.py:83-112): for every node the support_size nearest nodes by Euclidean
    distance, the first of them (the node itself) dropped; (N, support_size - 1) node ids in sorted order.
    The reference queries a BallTree on the original numbering and renumbers the result; distances do not
    depend on the numbering, so the sets agree wherever no two candidates tie at the edge of a support."""
    from scipy.spatial import cKDTree
    N = sorted_nodes.shape[0]
    assert 0 < support_size <= N, "support size must lie in [1, N] (updes/cloud.py:99-100)"
    _, nb = cKDTree(sorted_nodes).query(sorted_nodes, k=support_size)
    nb = np.asarray(nb, dtype=np.int64).reshape(N, support_size)
    return nb[:, 1:].copy()


def _support_mask(cloud: Cloud, supports, rows=None) -> np.ndarray:
    """(N, N) mask of the Phi columns each of the first N rows keeps: row i of an interior, Dirichlet, Neumann
    or Robin row (node a) keeps S(a); a periodic row (nodes a, b) keeps S(a) and S(b)
    (updes/assembly.py:20-32, 125-128, 169-258)."""
    N = cloud.N
    mask = np.zeros((N, N), dtype=bool)
    r = np.repeat(np.arange(N), supports.shape[1])
    mask[r, supports.reshape(-1)] = True
    if rows is not None:
        Ni = cloud.Ni
        for k in range(N - Ni):
            if rows.kind[k] in (ROW_PD, ROW_PN):
                a, b = rows.i1[k], rows.i2[k]
                mask[Ni + k] = False
                mask[Ni + k, supports[a]] = True
                mask[Ni + k, supports[b]] = True
    return mask


def jitter_coords(Nx: int, Ny: int, facet_types: dict, frac: float, seed: int) -> np.ndarray:
    """Grid coordinates (original-id order) with U(-frac*h, +frac*h) jitter on the nodes the
    reference jitters (type not in d/n/r, updes/cloud.py:441), h = min grid spacing.
    Seeded with ``numpy.random.default_rng(seed)`` — one (N, 2) draw."""
    xs = np.linspace(0.0, 1.0, Nx)
    ys = np.linspace(0.0, 1.0, Ny)
    h = min(xs[1] - xs[0], ys[1] - ys[0])
    rng = np.random.default_rng(seed)
    noise = rng.uniform(-frac * h, frac * h, size=(Nx * Ny, 2))
    base = square_cloud(Nx, Ny, facet_types)
    inv = {v: k for k, v in base.renumbering_map.items()}
    coords = np.zeros((Nx * Ny, 2))
    for g in range(Nx * Ny):
        i, j = divmod(g, Ny)
        coords[g] = (xs[i], ys[j])
        t = base.node_types[base.renumbering_map[g]]
        if t not in ("d", "n", "r"):
            coords[g] += noise[g]
    del inv
    return coords


# ---------------------------------------------------------------------------
# Boundary row descriptors (updes/assembly.py:141-362, operators.py:512-541)
# ---------------------------------------------------------------------------

ROW_D, ROW_N, ROW_R, ROW_PD, ROW_PN = 0, 1, 2, 3, 4


@dataclass
class BoundaryRows:
    kind: np.ndarray        # (Nb,) row type
    i1: np.ndarray          # evaluation node
    i2: np.ndarray          # partner node (periodic), else i1
    n1: np.ndarray          # (Nb, 2) normal used by the Φ part at i1
    n2: np.ndarray          # (Nb, 2) normal used by the Φ part at i2 (periodic flux rows)
    beta: np.ndarray        # (Nb,) Robin coefficient
    nP: np.ndarray          # (Nb, 2) normal used by the polynomial part


def robin_betas(cloud: Cloud, betas_by_facet: dict, compat: bool = True) -> dict:
    """Per-node Robin coefficient, updes/operators.py:512-541.

    ``betas_by_facet[f]`` is an array over ``cloud.facet_nodes[f]``.  The
    reference indexes it with ``i - node_ids[0]`` (operators.py:535), which
    equals the position in the facet when the facet's renumbered ids are
    contiguous; ``compat`` reproduces that index (clamped to the array).
    """
    out = {}
    for f, t in cloud.facet_types.items():
        if t != "r":
            continue
        ids = cloud.facet_nodes[f]
        b = np.broadcast_to(np.asarray(betas_by_facet.get(f, 0.0), dtype=np.float64), (len(ids),))
        for pos, i in enumerate(ids):
            ii = min(i - ids[0], len(ids) - 1) if compat else pos
            out[i] = float(b[ii])
    return out


def boundary_rows(cloud: Cloud, robin: dict, compat: bool = True) -> BoundaryRows:
    """Descriptors of the N - Ni boundary rows in the order the reference stacks them."""
    Ni, Nd, Nn, Nr = cloud.Ni, cloud.Nd, cloud.Nn, cloud.Nr
    son = cloud.sorted_outward_normals
    Nb = cloud.N - Ni
    kind = np.zeros(Nb, np.int32)
    i1 = np.zeros(Nb, np.int64)
    i2 = np.zeros(Nb, np.int64)
    n1 = np.zeros((Nb, 2))
    n2 = np.zeros((Nb, 2))
    beta = np.zeros(Nb)
    nP = np.zeros((Nb, 2))
    for i in range(Ni, Ni + Nd):                        # assembly.py:169-176, 283-287
        r = i - Ni
        kind[r], i1[r], i2[r] = ROW_D, i, i
    for i in range(Ni + Nd, Ni + Nd + Nn):              # assembly.py:178-190, 289-299
        r = i - Ni
        kind[r], i1[r], i2[r] = ROW_N, i, i
        n1[r] = son[i - Ni - Nd]
        nP[r] = cloud.outward_normals[i]
    for i in range(Ni + Nd + Nn, Ni + Nd + Nn + Nr):    # assembly.py:194-212, 301-315
        r = i - Ni
        kind[r], i1[r], i2[r] = ROW_R, i, i
        # bdΦ reads sorted_outward_normals[i-Ni-Nd-Nn] (assembly.py:206); bdP uses node i's normal
        n1[r] = son[i - Ni - Nd - Nn] if compat else cloud.outward_normals[i]
        nP[r] = cloud.outward_normals[i]
        beta[r] = robin.get(i, 0.0)
    half = sum(cloud.Np) // 2
    start = Ni + Nd + Nn + Nr
    row = start - Ni
    for npts in cloud.Np:                               # assembly.py:215-267, 317-359
        nc = npts // 2
        for k in range(nc):
            a, b = start + k, start + nc + k
            for rr, kd in ((row + k, ROW_PD), (row + k + half, ROW_PN)):
                kind[rr], i1[rr], i2[rr] = kd, a, b
                n1[rr] = son[a - Ni - Nd]
                n2[rr] = son[b - Ni - Nd]
                nP[rr] = cloud.outward_normals[a]
        row += nc
        start += npts
    return BoundaryRows(kind, i1, i2, n1, n2, beta, nP)


# ---------------------------------------------------------------------------
# Assembly
# ---------------------------------------------------------------------------

# Rows per block of the dense assemblies: bounds the temporaries (about 13 arrays of ROW_BLOCK x N FP64 per
# thread) at full size.
ROW_BLOCK = 256


def _row_blocks(nrows, fn, threads=None):
    """fn(r0, r1) over blocks of ROW_BLOCK rows on a thread pool (NumPy releases the GIL in its ufuncs)."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    blocks = [(r0, min(nrows, r0 + ROW_BLOCK)) for r0 in range(0, nrows, ROW_BLOCK)]
    threads = threads or min(16, os.cpu_count() or 1)
    if len(blocks) <= 1 or threads <= 1:
        for b in blocks:
            fn(*b)
        return
    with ThreadPoolExecutor(threads) as ex:
        for f in [ex.submit(fn, *b) for b in blocks]:
            f.result()


def _combine(t, w):
    """a φ + bx ∂xφ + by ∂yφ + wxx ∂xxφ + wyy ∂yyφ with per-row weights w (rows, 5)."""
    phi, gx, gy, hxx, hyy = t
    return (w[:, 0:1] * phi + w[:, 1:2] * gx + w[:, 2:3] * gy
            + w[:, 3:4] * hxx + w[:, 4:5] * hyy)


def assemble_K(cloud: Cloud, kind: str, param: float, max_degree: int, op_weights,
               rows: BoundaryRows, self_term: bool = False, supports=None) -> np.ndarray:
    """Augmented Kansa matrix K (n × n, n = N + M).

    Rows 0..Ni-1: interior operator rows opΦ | opP (assembly.py:93-137);
    rows Ni..N-1: boundary rows bdΦ | bdP (assembly.py:141-362);
    rows N..n-1: [Pᵀ | 0] (assembly.py:62-85).
    Φ-type blocks leave column i of row i at 0 (the support excludes the node
    itself, cloud.py:108-112) unless ``self_term``; periodic rows span all columns.
    ``op_weights``: (Ni, 5) = [a, bx, by, wxx, wyy] per interior node.
    """
    X = cloud.sorted_nodes
    N, Ni = cloud.N, cloud.Ni
    M = nb_monomials(max_degree)
    n = N + M
    K = np.zeros((n, n))
    W = np.asarray(op_weights, dtype=np.float64).reshape(Ni, 5)
    # interior Φ rows, in blocks of rows on a thread pool (elementwise arithmetic: the blocking changes nothing
    # but the size of the temporaries and the threads NumPy uses)
    def fill(r0, r1):
        dx = X[r0:r1, 0:1] - X[None, :, 0]
        dy = X[r0:r1, 1:2] - X[None, :, 1]
        K[r0:r1, :N] = _combine(rbf_terms(kind, param, dx, dy), W[r0:r1])
    _row_blocks(Ni, fill)
    if not self_term:
        K[np.arange(Ni), np.arange(Ni)] = 0.0
    for k in range(M):
        K[:Ni, N + k] = _combine([v[:, None] for v in monomial_terms(k, X[:Ni, 0], X[:Ni, 1])], W)[:, 0]
    # boundary rows
    Nb = N - Ni
    for r in range(Nb):
        row = Ni + r
        kd, a, b = rows.kind[r], rows.i1[r], rows.i2[r]
        ta = rbf_terms(kind, param, X[a, 0] - X[:, 0], X[a, 1] - X[:, 1])
        ma = [monomial_terms(k, X[a, 0], X[a, 1]) for k in range(M)]
        if kd == ROW_D:
            vals = ta[0].copy()
            pv = [m[0] for m in ma]
        elif kd == ROW_N:
            vals = ta[1] * rows.n1[r, 0] + ta[2] * rows.n1[r, 1]
            pv = [m[1] * rows.nP[r, 0] + m[2] * rows.nP[r, 1] for m in ma]
        elif kd == ROW_R:
            vals = rows.beta[r] * ta[0] + (ta[1] * rows.n1[r, 0] + ta[2] * rows.n1[r, 1])
            pv = [rows.beta[r] * m[0] + (m[1] * rows.nP[r, 0] + m[2] * rows.nP[r, 1]) for m in ma]
        else:
            tb = rbf_terms(kind, param, X[b, 0] - X[:, 0], X[b, 1] - X[:, 1])
            mb = [monomial_terms(k, X[b, 0], X[b, 1]) for k in range(M)]
            if kd == ROW_PD:
                vals = ta[0] - tb[0]
                pv = [m1[0] - m2[0] for m1, m2 in zip(ma, mb)]
            else:
                n1, n2 = rows.n1[r], rows.n2[r]
                vals = (ta[1] * n1[0] + ta[2] * n1[1]) - (tb[1] * (-n2[0]) + tb[2] * (-n2[1]))
                # bdP uses cloud.outward_normals by node id (assembly.py:343-355)
                pv = [(m1[1] * n1[0] + m1[2] * n1[1]) - (m2[1] * (-n2[0]) + m2[2] * (-n2[1]))
                      for m1, m2 in zip(ma, mb)]
        if kd in (ROW_D, ROW_N, ROW_R) and not self_term:
            vals[a] = 0.0
        K[row, :N] = vals
        K[row, N:] = pv
    # Pᵀ rows
    for k in range(M):
        K[N + k, :N] = monomial_terms(k, X[:, 0], X[:, 1])[0]
    if supports is not None:  # local supports: each row keeps the Phi columns of its support(s)
        K[:N, :N] *= _support_mask(cloud, supports, rows)
    return K


def assemble_A(cloud: Cloud, kind: str, param: float, max_degree: int,
               self_term: bool = False, supports=None) -> np.ndarray:
    """A = [[Φ, P], [Pᵀ, 0]] with Φ_ii = 0 (updes/assembly.py:10-85)."""
    X = cloud.sorted_nodes
    N = cloud.N
    M = nb_monomials(max_degree)
    A = np.zeros((N + M, N + M))

    def fill(r0, r1):
        A[r0:r1, :N] = rbf_terms(kind, param, X[r0:r1, 0:1] - X[None, :, 0], X[r0:r1, 1:2] - X[None, :, 1])[0]
    _row_blocks(N, fill)
    if not self_term:
        A[np.arange(N), np.arange(N)] = 0.0
    if supports is not None:
        A[:N, :N] *= _support_mask(cloud, supports)
    for k in range(M):
        p = monomial_terms(k, X[:, 0], X[:, 1])[0]
        A[:N, N + k] = p
        A[N + k, :N] = p
    return A


def assemble_q(cloud: Cloud, interior_rhs, bc_values: dict) -> np.ndarray:
    """q (N,): interior rhs then facet values scattered by node id; periodic facets 0
    (updes/assembly.py:434-485, operators.py:546-555)."""
    q = np.zeros(cloud.N)
    q[:cloud.Ni] = np.broadcast_to(np.asarray(interior_rhs, dtype=np.float64), (cloud.Ni,))
    for f, t in cloud.facet_types.items():
        ids = np.array(cloud.facet_nodes[f], dtype=np.int64)
        if t[0] == "p":
            q[ids] = 0.0
        else:
            q[ids] = np.broadcast_to(np.asarray(bc_values[f], dtype=np.float64), ids.shape)
    return q


# ---------------------------------------------------------------------------
# Solves
# ---------------------------------------------------------------------------

def solve_faithful(K: np.ndarray, A: np.ndarray, q: np.ndarray):
    """The reference's order of operations (updes/operators.py:602-616):
    B = diffMat · inv(A)[:, :N]; QR solve B u = q; c = inv(A) [u; 0]."""
    N = q.shape[0]
    diffMat = K[:N]
    invA = np.linalg.inv(A)
    B = (diffMat @ invA)[:, :N]
    Q, R = np.linalg.qr(B)
    u = sla.solve_triangular(R, Q.T @ q)
    c = invA @ np.concatenate([u, np.zeros(A.shape[0] - N)])
    return u, c, B


def solve_direct(K: np.ndarray, A: np.ndarray, q: np.ndarray):
    """One LU of K: K c = [q; 0], u = A[:N] c (algebraically identical)."""
    N = q.shape[0]
    b = np.concatenate([q, np.zeros(K.shape[0] - N)])
    c = sla.lu_solve(sla.lu_factor(K), b)
    u = A[:N] @ c
    return u, c


def eval_values(cloud: Cloud, kind: str, param: float, max_degree: int, c: np.ndarray,
                self_term: bool = False, supports=None) -> np.ndarray:
    """u = [Φ P] c at the nodes with Φ_ii = 0 (the product's regenerate-GEMV)."""
    return assemble_A(cloud, kind, param, max_degree, self_term, supports=supports)[:cloud.N] @ c


def value(xs, coeffs, centers, kind, param):
    """Field value at points ``xs`` (m, 2) from coefficients (updes/operators.py:118-147).
    Unlike the matrices, the sum runs over every center (φ(0) included)."""
    xs = np.atleast_2d(xs)
    N = centers.shape[0]
    lam, gam = coeffs[:N], coeffs[N:]
    phi = rbf_terms(kind, param, xs[:, 0:1] - centers[None, :, 0], xs[:, 1:2] - centers[None, :, 1])[0]
    out = np.nan_to_num(lam[None, :] * phi, posinf=0.0, neginf=0.0).sum(axis=1)
    for k in range(gam.shape[0]):
        out = out + gam[k] * monomial_terms(k, xs[:, 0], xs[:, 1])[0]
    return out


def gradient(xs, coeffs, centers, kind, param):
    """Field gradient at points ``xs`` (m, 2) (updes/operators.py:156-184)."""
    xs = np.atleast_2d(xs)
    N = centers.shape[0]
    lam, gam = coeffs[:N], coeffs[N:]
    t = rbf_terms(kind, param, xs[:, 0:1] - centers[None, :, 0], xs[:, 1:2] - centers[None, :, 1])
    gx = np.nan_to_num(lam[None, :] * t[1]).sum(axis=1)
    gy = np.nan_to_num(lam[None, :] * t[2]).sum(axis=1)
    for k in range(gam.shape[0]):
        m = monomial_terms(k, xs[:, 0], xs[:, 1])
        gx = gx + gam[k] * m[1]
        gy = gy + gam[k] * m[2]
    return np.stack([gx, gy], axis=-1)


def laplacian(xs, coeffs, centers, kind, param):
    """Field Laplacian at points ``xs`` (m, 2) (updes/operators.py:319-348): the trace of the Hessian of
    every kernel term (0 at r = 0) plus the monomials' second derivatives."""
    xs = np.atleast_2d(xs)
    N = centers.shape[0]
    lam, gam = coeffs[:N], coeffs[N:]
    t = rbf_terms(kind, param, xs[:, 0:1] - centers[None, :, 0], xs[:, 1:2] - centers[None, :, 1])
    out = np.nan_to_num(lam[None, :] * (t[3] + t[4])).sum(axis=1)
    for k in range(gam.shape[0]):
        m = monomial_terms(k, xs[:, 0], xs[:, 1])
        out = out + gam[k] * (m[3] + m[4])
    return out


def field_coefficients(cloud: Cloud, kind: str, param: float, max_degree: int, values, supports=None) -> np.ndarray:
    """c = inv(A) [values; 0] (updes/assembly.py:404-430)."""
    A = assemble_A(cloud, kind, param, max_degree, supports=supports)
    M = A.shape[0] - cloud.N
    return np.linalg.solve(A, np.concatenate([np.asarray(values, dtype=np.float64), np.zeros(M)]))
