"""Field helpers around the solve: values given at the nodes, quadrature, transfer between clouds and the
grid finite differences of the reference's Navier-Stokes demos (updes/operators.py:190-208, 211-291,
354-371, 381-509).

The RBF ones (``gradient_vals``, ``laplacian_vals``, ``integrate_field``) evaluate on the GPU through the
field kernels (``value``/``gradient``/``laplacian``); coefficients come from the FP64 interpolation solve
(``core_compute_coefficients``).  The others are index and nearest-neighbour work on the host, in NumPy.
Each reproduces the reference's results on its own inputs, including the quirks noted in the docstrings.
"""
from __future__ import annotations

import numpy as np

from .operators import compute_nb_monomials, core_compute_coefficients, gradient, laplacian, value_vec


def gradient_vals(x, field, cloud, rbf, max_degree):
    """Gradient at x of the field given by its nodal values (updes/operators.py:190-208)."""
    coeffs = core_compute_coefficients(field, cloud, rbf, compute_nb_monomials(max_degree))
    return gradient(x, coeffs, cloud.sorted_nodes, rbf)


def gradient_vals_vec(xs, field, cloud, rbf, max_degree):
    """``gradient_vals`` at the rows of xs (m, 2); one coefficient solve for all of them."""
    coeffs = core_compute_coefficients(field, cloud, rbf, compute_nb_monomials(max_degree))
    return gradient(np.asarray(xs, dtype=np.float64).reshape(-1, 2), coeffs, cloud.sorted_nodes, rbf)


def laplacian_vals(x, field, cloud, rbf, max_degree):
    """Laplacian at x of the field given by its nodal values (updes/operators.py:354-371)."""
    coeffs = core_compute_coefficients(field, cloud, rbf, compute_nb_monomials(max_degree))
    return laplacian(x, coeffs, cloud.sorted_nodes, rbf)


def laplacian_vals_vec(xs, field, cloud, rbf, max_degree):
    """``laplacian_vals`` at the rows of xs (m, 2)."""
    coeffs = core_compute_coefficients(field, cloud, rbf, compute_nb_monomials(max_degree))
    return laplacian(np.asarray(xs, dtype=np.float64).reshape(-1, 2), coeffs, cloud.sorted_nodes, rbf)


def integrate_field(field, cloud, rbf, max_degree=None):
    """Integral over the unit square of the field given by its coefficients: midpoint rule on the
    (Nx-1) x (Ny-1) grid cells, halved weights on the edges, quartered at the corners
    (updes/operators.py:381-450).  ``max_degree`` is unused, as in the reference.

    As in the reference, the top-left corner's value is taken at (1, 0) (its point variable is assigned
    but the bottom-right one is evaluated again), so a field that differs at (0, 1) and (1, 0) integrates
    as the reference does, not as the midpoint rule would."""
    from .cloud import SquareCloud
    assert isinstance(cloud, SquareCloud), "The cloud must be a SquareCloud instance"
    Nx, Ny = cloud.Nx, cloud.Ny
    centers = cloud.sorted_nodes
    area = (1 / (Nx - 1)) * (1 / (Ny - 1))
    qx = np.linspace(1 / (Nx - 1), 1 - 1 / (Nx - 1), Nx - 1)
    qy = np.linspace(1 / (Ny - 1), 1 - 1 / (Ny - 1), Ny - 1)
    # jnp.array(jnp.meshgrid(qx, qy)).reshape(nb_squares, 2): the stacked (2, Ny-1, Nx-1) grids read in C
    # order as (nb_squares, 2) pairs, which is what the reference evaluates
    inner = np.array(np.meshgrid(qx, qy)).reshape((Nx - 1) * (Ny - 1), 2)
    ey = np.linspace(1 / (Ny - 1), 1 - 1 / (Ny - 1), Ny - 2)
    ex = np.linspace(1 / (Nx - 1), 1 - 1 / (Nx - 1), Nx - 2)
    left = np.stack((np.zeros(Ny - 2), ey), axis=-1)
    right = np.stack((np.ones(Ny - 2), ey), axis=-1)
    bottom = np.stack((ex, np.zeros(Nx - 2)), axis=-1)
    top = np.stack((ex, np.ones(Nx - 2)), axis=-1)
    corners = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 0.0], [1.0, 1.0]])  # bl, br, "tl" (= br), tr
    pts = np.concatenate([inner, left, right, bottom, top, corners])
    vals = np.asarray(value_vec(pts, field, centers, rbf), dtype=np.float64)
    k = [len(inner), len(left), len(right), len(bottom), len(top)]
    o = np.cumsum([0] + k)
    s_in = np.sum(vals[o[0]:o[1]])
    s_edges = (np.sum(vals[o[1]:o[2]]) + np.sum(vals[o[2]:o[3]]) + np.sum(vals[o[3]:o[4]]) +
               np.sum(vals[o[4]:o[5]]))
    bl, br, tl, tr = vals[o[5]:o[5] + 4]
    return (s_in + 0.5 * s_edges + 0.25 * (bl + br + tl + tr)) * area


def interpolate_field(field, cloud1, cloud2):
    """The field given in cloud1's node numbering, in cloud2's (updes/operators.py:457-480): the two clouds
    hold the same nodes numbered differently (e.g. other facet types)."""
    assert cloud1.N == cloud2.N, "the two clouds do not contain the same number of nodes"
    field = np.asarray(field)
    N = cloud1.N
    new1 = np.array([cloud1.renumbering_map[g] for g in range(N)])  # original id -> cloud1's id
    new2 = np.array([cloud2.renumbering_map[g] for g in range(N)])
    field_orig = field[new1]                 # by original id
    orig_of_new2 = np.empty(N, dtype=np.int64)
    orig_of_new2[new2] = np.arange(N)        # cloud2's id -> original id
    return field_orig[orig_of_new2]


def _support(cloud, i):
    """Node i's support in the reference's order (nearest first); "max" supports: every other node."""
    X = cloud.sorted_nodes
    sup = getattr(cloud, "sorted_local_supports", None)
    if sup is not None:
        return np.asarray(sup[i], dtype=np.int64)
    d = np.linalg.norm(X - X[i], axis=1)
    order = np.argsort(d, kind="stable")
    return order[order != i]


def _opposite_closest(cloud, i, direction):
    """(closest node j of i's support with (x_j - x_i)/|x_j - x_i| within the cone dot(direction, .) + 1 <=
    0.1, its distance, the distance to the support's last node), the reference's neighbour rule (ties
    between equal distances go to the later node, as its loop keeps the last one); j is None when the cone
    holds no node."""
    X = cloud.sorted_nodes
    sup = _support(cloud, i)
    vec = X[sup] - X[i]
    norm = np.linalg.norm(vec, axis=1)
    ok = (vec / norm[:, None]) @ np.asarray(direction, dtype=np.float64) + 1.0 <= 1e-1
    if not np.any(ok):
        return None, None, float(norm[-1])
    cand = np.flatnonzero(ok)
    dmin = np.min(norm[cand])
    j = int(sup[cand[norm[cand] == dmin][-1]])
    return j, float(dmin), float(norm[-1])


def apply_neumann_conditions(field, boundary_conditions, cloud):
    """Each Neumann node takes the value of its closest support node opposite its outward normal
    (updes/operators.py:483-509); ``boundary_conditions`` is unused, as in the reference."""
    out = np.array(field, dtype=np.float64, copy=True)
    for f, t in cloud.facet_types.items():
        if t != "n":
            continue
        for i in cloud.facet_nodes[f]:
            j, _, _ = _opposite_closest(cloud, i, cloud.outward_normals[i])
            if j is None:
                raise ValueError(f"Neumann node {i}: no support node lies opposite its outward normal")
            out[i] = out[j]
    return out


def cartesian_gradient(node_id, field, cloud, clip_val=None):
    """One-sided finite-difference gradient at a node of a grid cloud (updes/operators.py:211-251).

    Reproduces the reference: each component is (field[i] - field[j]) / r with j the closest node in the
    opposite direction and r the distance to the *last* node of the support (the reference divides by its
    loop variable after the loop); if no node lies in the opposite direction of a component, the gradient
    computed so far is returned."""
    field = np.asarray(field, dtype=np.float64)
    i = int(node_id)
    g = np.zeros(2)
    for d, direction in ((0, (1.0, 0.0)), (1, (0.0, 1.0))):
        j, _, r_last = _opposite_closest(cloud, i, direction)
        if j is None:
            return g
        g[d] = (field[i] - field[j]) / r_last
    return np.clip(g, -clip_val, clip_val) if clip_val else g


def cartesian_gradient_vec(node_ids, field, cloud):
    """``cartesian_gradient`` of every node in node_ids, written at row node_id of a (len(node_ids), 2)
    array, as the reference does (updes/operators.py:254-259)."""
    node_ids = list(node_ids)
    grad = np.zeros((len(node_ids), 2))
    for node_id in node_ids:
        grad[node_id, :] = cartesian_gradient(node_id, field, cloud)
    return grad


def enforce_cartesian_gradient_neumann(field, grads, boundary_conditions, cloud, clip_val=None):
    """At each Neumann node both gradient components become (field[i] - field[j]) / |x_i - x_j|, j its
    closest support node opposite the outward normal (updes/operators.py:262-291: the reference writes the
    scalar into the node's whole row)."""
    field = np.asarray(field, dtype=np.float64)
    out = np.array(grads, dtype=np.float64, copy=True)
    for f, t in cloud.facet_types.items():
        if t != "n":
            continue
        for i in cloud.facet_nodes[f]:
            j, dist, _ = _opposite_closest(cloud, i, cloud.outward_normals[i])
            if j is None:
                raise ValueError(f"Neumann node {i}: no support node lies opposite its outward normal")
            out[i] = (field[i] - field[j]) / dist
    return np.clip(out, -clip_val, clip_val) if clip_val else out


def divergence_vec(xs, field, centers, rbf=None):
    """``divergence`` at the rows of xs (m, 2) of a vector field given by its two coefficient columns
    (updes/operators.py:314)."""
    from .operators import divergence
    return divergence(np.asarray(xs, dtype=np.float64).reshape(-1, 2), field, centers, rbf)


def dot_vec(a, b):
    """Row-wise dot products of two (m, d) arrays (updes/operators.py:778)."""
    return np.einsum("ij,ij->i", np.asarray(a), np.asarray(b))


def dot_mat(J, v):
    """Row-wise matrix-vector products J[i] @ v[i] of (m, p, d) and (m, d) arrays (updes/operators.py:779)."""
    return np.einsum("ipd,id->ip", np.asarray(J), np.asarray(v))


def zerofy_periodic_cond(boundary_conditions, cloud):
    """Zero values on the periodic facets, in place, as the solve does before it runs
    (updes/operators.py:546-555)."""
    for f, t in cloud.facet_types.items():
        if t[0] == "p":
            boundary_conditions[f] = np.zeros(len(cloud.facet_nodes[f]))
    return boundary_conditions


def duplicate_robin_coeffs(boundary_conditions, cloud):
    """(Robin coefficient per node, the boundary conditions with the Robin facets' values alone)
    (updes/operators.py:512-541).  A Robin facet given as (values, betas) spreads betas (an array, or a
    callable evaluated on the facet's nodes) over its nodes by position i - first node id, as the reference
    does, with the index clamped to the facet as the solver's compatibility mode does; a facet given without
    betas gets zeros."""
    from .operators import _eval_on_nodes
    robin, out = {}, {}
    for f, t in cloud.facet_types.items():
        bc = boundary_conditions[f]
        if t != "r":
            out[f] = bc
            continue
        ids = cloud.facet_nodes[f]
        if isinstance(bc, tuple):
            out[f], betas = bc[0], bc[1]
            if callable(betas):
                betas = _eval_on_nodes(betas, cloud.sorted_nodes[np.asarray(ids, dtype=np.int64)])
        else:
            out[f], betas = bc, np.zeros(len(ids))
        betas = np.broadcast_to(np.asarray(betas, dtype=np.float64), (len(ids),))
        for i in ids:
            robin[i] = float(betas[min(max(i - ids[0], 0), len(ids) - 1)])
    return robin, out
