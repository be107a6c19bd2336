"""Seeded synthetic workloads shaped like the benchmark configurations of the solve.

No dataset exists for these problems; each generator builds the clouds, operators
and boundary data from a seed, with the sizes and value distributions the
configurations name:

* ``readme_laplace``: Laplace on a 30 x 20 SquareCloud, South Neumann 0,
  West/East Dirichlet 0, North Dirichlet sin(pi x); r^3, degree 1 (the reference
  README example, demos/Laplace/00_laplace_with_rbf.py).
* ``poisson_manufactured``: Nx = Ny = nx, interior jitter U(-0.2h, 0.2h), all
  facets Dirichlet u* = sin(pi x) sin(pi y), rhs -2 pi^2 u*; r^3, degree 2.
* ``advection_bumps``: implicit-Euler advection-diffusion u/dt + v.grad u - kappa
  Lap u on Nx = Ny = 80 with v = (1, 0.5), kappa = 0.01, dt = 1e-3, Dirichlet 0,
  and R Gaussian bumps (centres U[0.3, 0.7]^2, widths U[0.05, 0.15]).
* ``boundary_control``: div(k grad u) on Nx = Ny = 100 with
  k = 1 + 0.5 sin(2 pi x) cos(2 pi y), the North facet's Dirichlet values as the
  control, other facets 0, J = mean over interior nodes of (u - u_t)^2 +
  1e-4 ||c||^2 with u_t = sinh(pi y) sin(pi x) / sinh(pi); r^5, degree 2.
* ``uneven_clouds``: independent Poisson problems on SquareClouds with Nx, Ny
  uniform in [10, 45], interior jitter U(-0.2h, 0.2h), each facet Dirichlet,
  Neumann or Robin at random (Robin beta U[0.5, 2], constant per facet), rhs an
  8-mode Fourier series sum_m a_m sin(pi k_m x + phi_m) sin(pi l_m y + psi_m) with
  a_m ~ N(0, 1), k_m, l_m in {1..4}, phases U[0, 2 pi); boundary values
  x^2 - y on every facet; Gaussian (eps U[1, 5]) and r^5 kernels alternating;
  degree 2.
"""
from __future__ import annotations

from functools import partial

import numpy as np

from .cloud import SquareCloud
from .operators import nodal_gradient, nodal_laplacian, nodal_value
from .rbf import gaussian, polyharmonic

FACETS = ("South", "West", "North", "East")


def readme_laplace():
    facets = {"South": "n", "West": "d", "North": "d", "East": "d"}
    cloud = SquareCloud(Nx=30, Ny=20, facet_types=facets)
    zero = lambda c: 0.0 * c[0]
    return dict(diff_operator=lambda x, center, rbf, monomial, fields: nodal_laplacian(x, center, rbf, monomial),
                rhs_operator=lambda x, centers, rbf, fields: 0.0 * x[0], cloud=cloud,
                boundary_conditions={"South": zero, "West": zero, "North": lambda c: np.sin(np.pi * c[0]),
                                     "East": zero},
                rbf=polyharmonic, max_degree=1)


def poisson_manufactured(nx=150, seed=0):
    facets = {f: "d" for f in FACETS}
    cloud = SquareCloud(Nx=nx, Ny=nx, facet_types=facets, jitter=(0.2, seed))
    ustar = lambda c: np.sin(np.pi * c[0]) * np.sin(np.pi * c[1])
    return dict(diff_operator=lambda x, center, rbf, monomial, fields: nodal_laplacian(x, center, rbf, monomial),
                rhs_operator=lambda x, centers, rbf, fields: -2 * np.pi ** 2 * np.sin(np.pi * x[0]) * np.sin(
                    np.pi * x[1]),
                cloud=cloud, boundary_conditions={f: ustar for f in FACETS}, rbf=polyharmonic, max_degree=2)


def advection_bumps(nx=80, nrhs=64, seed=0, dt=1e-3, kappa=0.01, velocity=(1.0, 0.5)):
    """(system dict without rhs, U0 (N, nrhs), dt): one implicit-Euler step solves
    (u/dt + v.grad u - kappa Lap u) u_new = u_old / dt."""
    facets = {f: "d" for f in FACETS}
    cloud = SquareCloud(Nx=nx, Ny=nx, facet_types=facets)

    def op(x, center, rbf, monomial, fields=None):
        g = nodal_gradient(x, center, rbf, monomial)
        return (nodal_value(x, center, rbf, monomial) / dt + velocity[0] * g[0] + velocity[1] * g[1]
                - kappa * nodal_laplacian(x, center, rbf, monomial))
    X = cloud.sorted_nodes
    rng = np.random.default_rng(seed)
    cen = rng.uniform(0.3, 0.7, (nrhs, 2))
    wid = rng.uniform(0.05, 0.15, nrhs)
    U0 = np.exp(-((X[:, None, 0] - cen[None, :, 0]) ** 2 + (X[:, None, 1] - cen[None, :, 1]) ** 2)
                / (2 * wid[None, :] ** 2))
    bcs = {f: np.zeros(len(cloud.facet_nodes[f])) for f in FACETS}
    return dict(diff_operator=op, cloud=cloud, boundary_conditions=bcs, rbf=polyharmonic, max_degree=1), U0, dt


def boundary_control(nx=100, ncontrols=32, seed=0):
    """(system dict for pde_solver_torch with fields [k, dk/dx, dk/dy], controls (ncontrols, nNorth),
    target u_t (N,))."""
    facets = {f: "d" for f in FACETS}
    cloud = SquareCloud(Nx=nx, Ny=nx, facet_types=facets)
    X = cloud.sorted_nodes
    k = 1 + 0.5 * np.sin(2 * np.pi * X[:, 0]) * np.cos(2 * np.pi * X[:, 1])
    kx = np.pi * np.cos(2 * np.pi * X[:, 0]) * np.cos(2 * np.pi * X[:, 1])
    ky = -np.pi * np.sin(2 * np.pi * X[:, 0]) * np.sin(2 * np.pi * X[:, 1])

    def op(x, center, rbf, monomial, fields):
        g = nodal_gradient(x, center, rbf, monomial)
        return fields[0] * nodal_laplacian(x, center, rbf, monomial) + fields[1] * g[0] + fields[2] * g[1]
    rng = np.random.default_rng(seed)
    controls = rng.standard_normal((ncontrols, len(cloud.facet_nodes["North"])))
    ut = np.sinh(np.pi * X[:, 1]) * np.sin(np.pi * X[:, 0]) / np.sinh(np.pi)
    bcs = {f: np.zeros(len(cloud.facet_nodes[f])) for f in FACETS}
    sysd = dict(diff_operator=op, rhs_operator=lambda x, centers, rbf, fields: 0.0 * x[0], cloud=cloud,
                boundary_conditions=bcs, rbf=partial(polyharmonic, a=2), max_degree=2)
    return sysd, [k, kx, ky], controls, ut


def uneven_clouds(count=512, seed=0):
    rng = np.random.default_rng(seed)
    systems = []
    for i in range(count):
        nx, ny = rng.integers(10, 46, size=2)
        kinds = rng.choice(["d", "n", "r"], size=4)
        if "d" not in kinds:  # keep the problem well posed: at least one Dirichlet facet
            kinds[rng.integers(0, 4)] = "d"
        facets = dict(zip(FACETS, kinds))
        cloud = SquareCloud(Nx=int(nx), Ny=int(ny), facet_types=facets, jitter=(0.2, int(rng.integers(1 << 30))))
        a = rng.standard_normal(8)
        km, lm = rng.integers(1, 5, size=8), rng.integers(1, 5, size=8)
        ph, ps = rng.uniform(0, 2 * np.pi, 8), rng.uniform(0, 2 * np.pi, 8)

        def rhs(x, centers, rbf, fields, a=a, km=km, lm=lm, ph=ph, ps=ps):
            return sum(a[m] * np.sin(np.pi * km[m] * x[0] + ph[m]) * np.sin(np.pi * lm[m] * x[1] + ps[m])
                       for m in range(8))
        g = lambda c: c[0] ** 2 - c[1]
        bcs = {}
        for f, kd in facets.items():
            bcs[f] = (g, (lambda c, b=rng.uniform(0.5, 2.0): b + 0.0 * c[0])) if kd == "r" else g
        rbf = partial(gaussian, eps=float(rng.uniform(1, 5))) if i % 2 == 0 else partial(polyharmonic, a=2)
        systems.append(dict(diff_operator=lambda x, center, rbf, monomial, fields: nodal_laplacian(x, center, rbf,
                                                                                                    monomial),
                            rhs_operator=rhs, cloud=cloud, boundary_conditions=bcs, rbf=rbf, max_degree=2))
    return systems
