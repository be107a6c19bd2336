"""Golden-case descriptions shared by the fixture generator and the tests.

Each case is written once, array-library agnostic (``xp`` is numpy for the
oracle and the product, or the jax stand-in when the reference is run), so the
reference run and every checker see the same problem.
"""
from __future__ import annotations

import numpy as np

# --- boundary-value and rhs functions of (xp, x, y) -------------------------


def zero(xp, x, y):
    return 0.0 * x


def one(xp, x, y):
    return 0.0 * x + 1.0


def sinpix(xp, x, y):
    return xp.sin(xp.pi * x)


def sinsin(xp, x, y):
    return xp.sin(xp.pi * x) * xp.sin(xp.pi * y)


def poisson_rhs(xp, x, y):
    return -2.0 * xp.pi ** 2 * xp.sin(xp.pi * x) * xp.sin(xp.pi * y)


def xsq(xp, x, y):
    return x * x


def ylin(xp, x, y):
    return 0.5 * y - 0.25


def xy(xp, x, y):
    return x * y


def beta2(xp, x, y):
    return 0.0 * x + 2.0


def beta_var(xp, x, y):
    return 0.0 * x + 0.75


FUNCS = {f.__name__: f for f in (zero, one, sinpix, sinsin, poisson_rhs, xsq, ylin, xy, beta2, beta_var)}

# --- operators ---------------------------------------------------------------
# Each operator is described by its per-interior-node weights on
# [value, d/dx, d/dy, d2/dx2, d2/dy2] as a function of (x, y, fields (F, m)).

ADV_DT, ADV_VEL, ADV_K = 1e-3, (1.0, 0.5), 0.01


def op_weights(op: str, x, y, fields):
    z = np.zeros_like(x)
    if op == "laplacian":
        return np.stack([z, z, z, z + 1.0, z + 1.0], axis=-1)
    if op == "advdiff":
        return np.stack([z + 1.0 / ADV_DT, z + ADV_VEL[0], z + ADV_VEL[1], z - ADV_K, z - ADV_K], axis=-1)
    if op == "kgrad":           # k Δu + ∇k·∇u with fields [k, kx, ky]
        k, kx, ky = fields[0], fields[1], fields[2]
        return np.stack([z, kx, ky, k, k], axis=-1)
    if op == "darcy":           # nodal_div_grad with (perm, perm) + fields[1]·value
        perm, s = fields[0], fields[1]
        return np.stack([s, z, z, perm, perm], axis=-1)
    if op == "helmholtz_x":     # Δu + (1 + x y) u
        return np.stack([1.0 + x * y, z, z, z + 1.0, z + 1.0], axis=-1)
    raise ValueError(op)


def make_fields(case, nodes):
    """Per-node diff_args fields (F, N) for a case, from the sorted node coordinates."""
    x, y = nodes[:, 0], nodes[:, 1]
    if case.get("fields") == "kfield":
        k = 1.0 + 0.5 * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
        kx = 0.5 * 2 * np.pi * np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y)
        ky = -0.5 * 2 * np.pi * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)
        return np.stack([k, kx, ky])
    if case.get("fields") == "perm":
        return np.stack([1.0 + x * x + 0.5 * y, 0.3 + 0.1 * x])
    return None


def make_rhs_field(case, nodes):
    """Nodal values passed as rhs_args (advection-diffusion: a Gaussian bump)."""
    if case.get("rhs") != "value_over_dt":
        return None
    x, y = nodes[:, 0], nodes[:, 1]
    return np.exp(-((x - 0.45) ** 2 + (y - 0.55) ** 2) / (2 * 0.1 ** 2))


CASES = {
    # the reference README example: Laplace, S=Neumann, W/E/N Dirichlet, r^3, degree 1
    "readme_laplace_30x20": dict(Nx=30, Ny=20, facets={"South": "n", "West": "d", "North": "d", "East": "d"},
                                 rbf=("polyharmonic", 1), max_degree=1, jitter=None, op="laplacian",
                                 bc={"South": "zero", "West": "zero", "North": "sinpix", "East": "zero"},
                                 rhs="zero"),
    # miniature of the Poisson manufactured-solution workload (jittered, degree 2)
    "poisson_jitter_11x11": dict(Nx=11, Ny=11, facets={"South": "d", "West": "d", "North": "d", "East": "d"},
                                 rbf=("polyharmonic", 1), max_degree=2, jitter=(0.2, 7), op="laplacian",
                                 bc={"South": "sinsin", "West": "sinsin", "North": "sinsin", "East": "sinsin"},
                                 rhs="poisson_rhs"),
    # Gaussian (diagonal quirk), Neumann + Robin together (Robin normal quirk), degree 2
    "gaussian_dnr_9x8": dict(Nx=9, Ny=8, facets={"South": "n", "West": "n", "North": "d", "East": "r"},
                             rbf=("gaussian", 3.0), max_degree=2, jitter=(0.2, 3), op="helmholtz_x",
                             bc={"South": "zero", "West": "ylin", "North": "xsq", "East": ("ylin", "beta2")},
                             rhs="one"),
    # variable-coefficient operator through fields (boundary-control workload), r^5
    "kgrad_fields_10x10": dict(Nx=10, Ny=10, facets={"South": "d", "West": "d", "North": "d", "East": "d"},
                               rbf=("polyharmonic", 2), max_degree=2, jitter=None, op="kgrad",
                               fields="kfield",
                               bc={"South": "zero", "West": "zero", "North": "sinpix", "East": "zero"},
                               rhs="zero"),
    # nodal_div_grad (tuple args) + field-weighted value, multiquadric
    "darcy_mq_8x8": dict(Nx=8, Ny=8, facets={"South": "d", "West": "d", "North": "d", "East": "d"},
                         rbf=("multiquadric", 1.5), max_degree=1, jitter=(0.2, 11), op="darcy", fields="perm",
                         bc={"South": "zero", "West": "xy", "North": "xsq", "East": "ylin"}, rhs="xy"),
    # advection-diffusion with the rhs built from nodal values (rhs_args → coefficients)
    "advdiff_rhsargs_9x9": dict(Nx=9, Ny=9, facets={"South": "d", "West": "d", "North": "d", "East": "d"},
                                rbf=("polyharmonic", 1), max_degree=1, jitter=(0.2, 5), op="advdiff",
                                bc={"South": "zero", "West": "zero", "North": "zero", "East": "zero"},
                                rhs="value_over_dt"),
    # periodic North/South pair + inverse multiquadric
    "periodic_imq_8x7": dict(Nx=8, Ny=7, facets={"North": "p1", "South": "p1", "West": "d", "East": "d"},
                             rbf=("inverse_multiquadric", 2.0), max_degree=1, jitter=None, op="laplacian",
                             bc={"North": "zero", "South": "zero", "West": "zero", "East": "one"},
                             rhs="one"),
    # thin plate spline, degree 4 (all 15 monomials), Robin without Neumann
    "thinplate_deg4_8x8": dict(Nx=8, Ny=8, facets={"South": "d", "West": "r", "North": "d", "East": "d"},
                               rbf=("thin_plate", 1), max_degree=4, jitter=(0.2, 13), op="helmholtz_x",
                               bc={"South": "xsq", "West": ("zero", "beta_var"), "North": "one", "East": "xy"},
                               rhs="sinsin"),
}

# Local supports (support_size an int, updes/cloud.py:83-112): each node's support is its support_size - 1
# nearest other nodes, and every Phi block keeps only those columns (the reference's "RBF-FD" clouds).  The
# clouds are jittered, so no two candidates tie at the edge of a support.
LOCAL_CASES = {
    "poisson_local_12x12": dict(Nx=12, Ny=12, facets={"South": "d", "West": "d", "North": "d", "East": "d"},
                                rbf=("polyharmonic", 1), max_degree=1, jitter=(0.2, 21), op="laplacian",
                                bc={"South": "sinsin", "West": "sinsin", "North": "sinsin", "East": "sinsin"},
                                rhs="poisson_rhs", support=20),
    "gaussian_dnr_local_11x10": dict(Nx=11, Ny=10, facets={"South": "n", "West": "n", "North": "d", "East": "r"},
                                     rbf=("gaussian", 3.0), max_degree=2, jitter=(0.2, 23), op="helmholtz_x",
                                     bc={"South": "zero", "West": "ylin", "North": "xsq", "East": ("ylin", "beta2")},
                                     rhs="one", support=16),
    "kgrad_local_10x10": dict(Nx=10, Ny=10, facets={"South": "d", "West": "d", "North": "d", "East": "d"},
                              rbf=("polyharmonic", 2), max_degree=2, jitter=(0.2, 25), op="kgrad", fields="kfield",
                              bc={"South": "zero", "West": "zero", "North": "sinpix", "East": "zero"},
                              rhs="zero", support=22),
    "periodic_local_10x9": dict(Nx=10, Ny=9, facets={"North": "p1", "South": "p1", "West": "d", "East": "d"},
                                rbf=("multiquadric", 1.5), max_degree=1, jitter=(0.2, 27), op="laplacian",
                                bc={"North": "zero", "South": "zero", "West": "zero", "East": "one"},
                                rhs="one", support=12),
}
LOCAL_ADJOINT_CASE = "kgrad_local_10x10"

# Cases whose matrices are stored in full (the others store a row subset + row checksums).
FULL_MATRIX_MAX_N = 150
ROW_STRIDE = 7

# Adjoint golden: boundary control on the kgrad case; gradients of
# J = mean_interior (u - u_t)^2 + 1e-4 ||c||^2 with respect to the North values c and the fields.
ADJOINT_CASE = "kgrad_fields_10x10"
ADJOINT_REG = 1e-4


def adjoint_target(xp, x, y):
    return xp.sinh(xp.pi * y) * xp.sin(xp.pi * x) / xp.sinh(xp.pi)


def adjoint_control(n):
    return np.random.default_rng(2024).standard_normal(n)


def grid_coords(case) -> np.ndarray:
    """Node coordinates in ORIGINAL global-id order (id = i*Ny + j), optionally jittered.

    Jitter follows the reference's rule (updes/cloud.py:441): every node whose
    type is not d/n/r moves (interior and periodic nodes), here by
    U(-frac*h, +frac*h) per coordinate with h the smaller grid spacing, drawn
    as one (N, 2) block from ``numpy.random.default_rng(seed)``.
    """
    Nx, Ny = case["Nx"], case["Ny"]
    xs = np.linspace(0.0, 1.0, Nx)
    ys = np.linspace(0.0, 1.0, Ny)
    ii, jj = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    coords = np.stack([xs[ii], ys[jj]], axis=-1)
    if case.get("jitter") is None:
        return coords
    frac, seed = case["jitter"]
    h = min(xs[1] - xs[0], ys[1] - ys[0])
    noise = np.random.default_rng(seed).uniform(-frac * h, frac * h, size=coords.shape)
    f = case["facets"]
    ftype = np.where(jj == Ny - 1, f["North"], np.where(jj == 0, f["South"], np.where(
        ii == Nx - 1, f["East"], np.where(ii == 0, f["West"], "i"))))
    move = ~np.isin(ftype, ["d", "n", "r"])
    coords[move] += noise[move]
    return coords


# --- coupled systems solved with pde_multi_solver (updes/operators.py:686-771) -------------------------
# Two fields (u, v) on one cloud; every sweep solves each field's PDE with the previous sweep's values of
# both fields as its leading diff_args, and rhs_args fixed at the old time level.
#  "grayscott": one implicit step of Gray-Scott reaction-diffusion as in the reference's demo
#     (demos/Gray-Scott/002_gray_scott_ode.py): operators u and v themselves (nodal_value), right-hand
#     sides Du Δu_old - u_old v~^2 + F (1 - u_old) and Dv Δv_old + u~ v_old^2 - (F + k) v_old.
#  "advect": Picard-linearised Burgers (demos/Burgers/00_burgers.py with u u_x written as u~ u_x):
#     operators u/dt + u~ u_x + v~ u_y and v/dt + u~ v_x + v~ v_y, right-hand sides u_old/dt, v_old/dt.
GS_DU, GS_DV, GS_F, GS_K = 0.2097, 0.105, 0.03, 0.062
BURGERS_DT = 0.05

MULTI_CASES = {
    "multi_grayscott_10x10": dict(Nx=10, Ny=10, facets={"South": "d", "West": "d", "North": "d", "East": "d"},
                                  rbf=("polyharmonic", 1), max_degree=1, jitter=None, kind="grayscott",
                                  nb_iters=3),
    "multi_advect_9x9": dict(Nx=9, Ny=9, facets={"South": "d", "West": "d", "North": "d", "East": "d"},
                             rbf=("polyharmonic", 1), max_degree=1, jitter=(0.2, 17), kind="advect", nb_iters=4),
}


def multi_initial(case, nodes):
    """Initial (old-time) values of the two fields at the sorted nodes: smooth bumps, zero on the boundary
    for the advection case."""
    x, y = nodes[:, 0], nodes[:, 1]
    bump = np.exp(-((x - 0.4) ** 2 + (y - 0.55) ** 2) / 0.02)
    if case["kind"] == "grayscott":
        return 0.95 - 0.5 * bump, 0.05 + 0.5 * bump
    s = np.sin(np.pi * x) * np.sin(np.pi * y)
    return 0.8 * s * (1.0 + 0.5 * bump), 0.4 * s * (1.0 - 0.3 * bump)


# --- Gmsh cloud (updes/cloud.py:520-734) on the synthetic mesh written by make_msh.py -----------------
GMSH_CASE = dict(mesh="dshape.msh", facets={"Bottom": "d", "Right": "n", "Top": "r", "Left": "d"},
                 rbf=("polyharmonic", 1), max_degree=1, op="laplacian",
                 bc={"Bottom": "sinsin", "Right": "xy", "Top": ("ylin", "beta2"), "Left": "zero"}, rhs="poisson_rhs")


# Field helpers around the solve (updes/operators.py:190-208, 211-291, 354-371, 381-509).  The integral
# case is the reference's own unit test problem (updes/tests/test_integrals.py: 12 x 12 Dirichlet cloud,
# r^11 (polyharmonic a = 5), degree 3, s = x^2 / (1 + y^2), whose integral over the unit square is pi/12),
# plus a 12 x 9 jittered cloud on which the reference's quadrature points are not the cell centres; the
# interpolation case is its test_interpolation.py problem (8 x 8, two facet assignments, field = node id).
FIELD_INTEGRAL_CASES = {
    "integral_12x12": dict(Nx=12, Ny=12, facets=dict(North="d", South="d", East="d", West="d"), jitter=None,
                           rbf=("polyharmonic", 5), max_degree=3),
    "integral_12x9_jitter": dict(Nx=12, Ny=9, facets=dict(North="d", South="n", East="d", West="r"),
                                 jitter=(0.2, 41), rbf=("polyharmonic", 5), max_degree=3),
}
FIELD_INTERP_CASE = dict(Nx=8, Ny=8, facets1=dict(South="n", West="d", North="n", East="d"),
                         facets2=dict(South="d", West="n", North="d", East="n"))
FIELD_FD_CASE = dict(Nx=9, Ny=7, facets=dict(North="n", South="n", East="d", West="n"), jitter=(0.15, 7))
FIELD_FD_SUPPORT = 12  # the grid finite differences again on 12-nearest-node supports
FIELD_EVAL_POINTS = np.array([[0.31, 0.42], [0.5, 0.5], [0.05, 0.9], [0.77, 0.13], [1.0, 0.25], [0.0, 0.0],
                              [0.62, 0.99]])


def field_s(X):
    """s = x^2 / (1 + y^2) (updes/tests/test_integrals.py)."""
    return X[:, 0] ** 2 / (1 + X[:, 1] ** 2)
