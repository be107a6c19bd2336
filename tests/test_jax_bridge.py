"""The JAX bridge (custom VJP over DLPack): needs JAX and a GPU, neither of which this environment has,
so it is skipped here and runs wherever both exist."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_jax_grad_matches_torch_adjoint():
    jax = pytest.importorskip("jax")
    import jax.numpy as jnp
    import torch

    import updes_gb300 as U
    from updes_gb300.adjoint import pde_solver_torch
    from updes_gb300.jax_bridge import pde_solver_jax

    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    cl = U.SquareCloud(Nx=10, Ny=10, facet_types=facets)
    op = lambda x, center, rbf, monomial, fields: U.nodal_laplacian(x, center, rbf, monomial)
    rhs = lambda x, centers, rbf, fields: 0.0 * x[0]
    nN = len(cl.facet_nodes["North"])
    tmpl = {f: np.zeros(len(cl.facet_nodes[f])) for f in facets}
    f = pde_solver_jax(op, rhs, cl, U.polyharmonic, 1, tmpl)
    c0 = np.random.default_rng(0).standard_normal(nN)

    def loss(c):
        vals, _ = f({"North": c}, ())
        return jnp.mean(vals ** 2)
    gj = np.asarray(jax.grad(loss)(jnp.asarray(c0)))
    ct = torch.tensor(c0, device="cuda", requires_grad=True)
    bcs = dict(tmpl)
    bcs["North"] = ct
    vals, _ = pde_solver_torch(op, rhs, cl, bcs, U.polyharmonic, 1)
    torch.mean(vals ** 2).backward()
    assert np.allclose(gj, ct.grad.cpu().numpy(), rtol=1e-10, atol=1e-14)
