"""Oracle results at the benchmark configurations' own sizes (FP64, NumPy/SciPy).

Usage:

    python tests/golden/make_fullsize.py [poisson] [control] [advection] [--faithful]

The small golden cases pin the oracle to the reference's own outputs; this
script runs that pinned oracle (``oracle/updes_np.py``) at the sizes the GPU
is benchmarked on, so the GPU tests can compare against an FP64 CPU result of
the same problem instead of against another GPU path:

* ``poisson``   (``full_poisson_150.npz``): the N = 22,500 Poisson
  manufactured-solution system (SquareCloud 150 x 150, interior jitter
  U(-0.2h, 0.2h) with seed 0, all facets Dirichlet u* = sin(pi x) sin(pi y),
  rhs -2 pi^2 u*, r^3, degree 2).  vals/coeffs of the direct LU of the Kansa
  matrix; with ``--faithful`` also the reference's own order of operations
  (inv -> GEMM -> QR -> inv, updes/operators.py:602-618), which takes minutes.
* ``control``   (``full_control_100.npz``): the N = 10,000 boundary-control
  problem (div(k grad u), r^5, degree 2) for the first of its 32 seeded
  controls: J, dJ/dc and dJ/d(fields) by a dense FP64 adjoint
  (lambda = K^-T g on SciPy's LU, dJ/dW_i = -lambda_i (D c)_i), twice: on
  the plain LU of K, on the LU of K equilibrated by powers of two, and on
  the LU of K with every entry moved by up to one unit in the last place.
  This r^5 system is so ill-conditioned that these backward-stable FP64
  solves disagree at the 1e-3 to 1e-2 level; that distance is the problem's
  FP64 floor, against which a GPU result is judged.
* ``advection`` (``full_advection_80.npz``): the first implicit-Euler step of
  the N = 6,400 advection-diffusion problem for its 64 seeded bumps: the
  values of 8 columns in full and, for all 64, their norms and their dot
  products with a seeded random vector.

The problems are built by the oracle alone (its cloud, rows and weights) with
the same seeds as ``updes_gb300.workloads``; the GPU tests rebuild them
through the product.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np
import scipy.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import updes_np as O  # noqa: E402

FACETS = {"South": "d", "West": "d", "North": "d", "East": "d"}


def _laplacian_weights(Ni):
    W = np.zeros((Ni, 5))
    W[:, 3:] = 1.0
    return W


def poisson(faithful: bool):
    t0 = time.time()
    nx = 150
    coords = O.jitter_coords(nx, nx, FACETS, 0.2, 0)
    cl = O.square_cloud(nx, nx, FACETS, coords=coords)
    X = cl.sorted_nodes
    us = np.sin(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1])
    K = O.assemble_K(cl, "polyharmonic", 1, 2, _laplacian_weights(cl.Ni), O.boundary_rows(cl, {}))
    A = O.assemble_A(cl, "polyharmonic", 1, 2)
    q = np.where(np.arange(cl.N) < cl.Ni, -2 * np.pi ** 2 * us, us)
    t1 = time.time()
    u, c = O.solve_direct(K, A, q)
    t2 = time.time()
    out = dict(vals=u, coeffs=c, sorted_nodes_digest=np.array([X.sum(), (X * X).sum()]),
               seconds=np.array([t1 - t0, t2 - t1]))
    print(f"poisson: assembly {t1 - t0:.1f} s, direct LU {t2 - t1:.1f} s, "
          f"rel err vs u* {np.linalg.norm(u - us) / np.linalg.norm(us):.3e}", flush=True)
    if faithful:
        uf, cf, _ = O.solve_faithful(K, A, q)
        t3 = time.time()
        out.update(vals_faithful=uf, coeffs_faithful=cf, seconds_faithful=np.array(t3 - t2))
        print(f"poisson: faithful {t3 - t2:.1f} s, faithful vs direct "
              f"{np.linalg.norm(uf - u) / np.linalg.norm(u):.3e}", flush=True)
    np.savez_compressed(os.path.join(HERE, "full_poisson_150.npz"), **out)


def control():
    t0 = time.time()
    nx = 100
    cl = O.square_cloud(nx, nx, FACETS)
    X = cl.sorted_nodes
    N, Ni = cl.N, cl.Ni
    x, y = X[:, 0], X[:, 1]
    k = 1 + 0.5 * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y)
    kx = np.pi * np.cos(2 * np.pi * x) * np.cos(2 * np.pi * y)
    ky = -np.pi * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)
    ctl = np.random.default_rng(0).standard_normal((32, len(cl.facet_nodes["North"])))[0]
    ut = np.sinh(np.pi * y) * np.sin(np.pi * x) / np.sinh(np.pi)
    rows = O.boundary_rows(cl, {})
    W = np.stack([0 * x, kx, ky, k, k], axis=-1)[:Ni]
    K = O.assemble_K(cl, "polyharmonic", 2, 2, W, rows)
    A = O.assemble_A(cl, "polyharmonic", 2, 2)
    M = K.shape[0] - N
    north = np.asarray(cl.facet_nodes["North"], dtype=np.int64)
    q = np.zeros(N)
    q[north] = ctl
    b = np.concatenate([q, np.zeros(M)])
    D = []
    for kk in range(1, 5):
        e = np.zeros((Ni, 5))
        e[:, kk] = 1.0
        D.append(O.assemble_K(cl, "polyharmonic", 2, 2, e, rows)[:Ni])

    def adjoint(solve, solve_t):
        c = solve(b)
        u = A[:N] @ c
        J = np.mean((u[:Ni] - ut[:Ni]) ** 2) + 1e-4 * np.sum(ctl ** 2)
        dJdu = np.zeros(N)
        dJdu[:Ni] = 2.0 * (u[:Ni] - ut[:Ni]) / Ni
        lam = solve_t(A[:N].T @ dJdu)
        dW = np.zeros((Ni, 5))
        for kk in range(1, 5):
            dW[:, kk] = -lam[:Ni] * (D[kk - 1] @ c)
        dF = np.zeros((3, N))
        dF[0, :Ni] = dW[:, 3] + dW[:, 4]
        dF[1, :Ni] = dW[:, 1]
        dF[2, :Ni] = dW[:, 2]
        return J, lam[north] + 2e-4 * ctl, dF, u

    # the plain LU of K, and the LU of K equilibrated by powers of two (rows, then columns, as the GPU path
    # does): two backward-stable FP64 solves whose distance is this problem's FP64 floor
    lu = sla.lu_factor(K)
    J, dJ_dc, dJ_dfields, u = adjoint(lambda v: sla.lu_solve(lu, v), lambda v: sla.lu_solve(lu, v, trans=1))
    r = 2.0 ** np.round(-np.log2(np.abs(K).max(1)))
    cs = 2.0 ** np.round(-np.log2(np.abs(K * r[:, None]).max(0)))
    lue = sla.lu_factor(K * r[:, None] * cs[None, :])
    Je, dce, dFe, ue = adjoint(lambda v: cs * sla.lu_solve(lue, r * v), lambda v: r * sla.lu_solve(lue, cs * v, trans=1))
    # and the plain LU of K with every entry moved by up to one unit in the last place (seeded): two FP64
    # assemblies of the same matrix (closed forms evaluated in a different order) differ by that much
    Kp = K * (1.0 + np.random.default_rng(2).uniform(-1.0, 1.0, K.shape) * 2.0 ** -53)
    lup = sla.lu_factor(Kp)
    Jp, dcp, dFp, up = adjoint(lambda v: sla.lu_solve(lup, v), lambda v: sla.lu_solve(lup, v, trans=1))
    np.savez_compressed(os.path.join(HERE, "full_control_100.npz"), control=ctl, J=np.array(J), dJ_dc=dJ_dc,
                        dJ_dfields=dJ_dfields, vals=u, J_eq=np.array(Je), dJ_dc_eq=dce, dJ_dfields_eq=dFe,
                        vals_eq=ue, J_ulp=np.array(Jp), dJ_dc_ulp=dcp, dJ_dfields_ulp=dFp, vals_ulp=up)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    for name, (Jx, dcx, dFx, ux) in (("equilibrated LU", (Je, dce, dFe, ue)), ("entries moved by 1 ulp", (Jp, dcp, dFp, up))):
        print(f"control: J = {J:.6e}; plain LU vs {name}: J {abs(J - Jx) / abs(J):.2e}, vals {rel(ux, u):.2e}, "
              f"dJ/dc {rel(dcx, dJ_dc):.2e}, dJ/dfields {rel(dFx, dJ_dfields):.2e}", flush=True)
    print(f"control: {time.time() - t0:.1f} s", flush=True)


def advection():
    t0 = time.time()
    nx, R, dt, kappa, vel = 80, 64, 1e-3, 0.01, (1.0, 0.5)
    cl = O.square_cloud(nx, nx, FACETS)
    X = cl.sorted_nodes
    N, Ni = cl.N, cl.Ni
    rng = np.random.default_rng(0)
    cen = rng.uniform(0.3, 0.7, (R, 2))
    wid = rng.uniform(0.05, 0.15, R)
    U0 = np.exp(-((X[:, None, 0] - cen[None, :, 0]) ** 2 + (X[:, None, 1] - cen[None, :, 1]) ** 2)
                / (2 * wid[None, :] ** 2))
    W = np.tile([1.0 / dt, vel[0], vel[1], -kappa, -kappa], (Ni, 1))
    K = O.assemble_K(cl, "polyharmonic", 1, 1, W, O.boundary_rows(cl, {}))
    A = O.assemble_A(cl, "polyharmonic", 1, 1)
    M = K.shape[0] - N
    Q = np.zeros((N + M, R))
    Q[:Ni] = U0[:Ni] / dt
    C = sla.lu_solve(sla.lu_factor(K), Q)
    U1 = A[:N] @ C
    w = np.random.default_rng(1).standard_normal(N)
    np.savez_compressed(os.path.join(HERE, "full_advection_80.npz"), U1_cols=U1[:, :8], col_norms=np.linalg.norm(U1, axis=0),
                        col_dots=w @ U1, probe=w)
    print(f"advection: {time.time() - t0:.1f} s", flush=True)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    which = args or ["poisson", "control", "advection"]
    if "advection" in which:
        advection()
    if "control" in which:
        control()
    if "poisson" in which:
        poisson("--faithful" in sys.argv)
