"""GPU: the JAX bridge's own logic (argument routing, the forward tape, the mapping of the backward pass's
gradients back to boundary values and fields) under a minimal stand-in for the three JAX entry points it
uses: ``jax.custom_vjp`` (fwd/bwd registration), ``jax.dlpack.from_dlpack`` and ``jax.numpy.zeros_like``.
The stand-in's "JAX arrays" are torch tensors, so DLPack is the identity.  What this cannot check is JAX
itself (tracing, its DLPack import, ``jax.grad``'s handling of the custom rule): JAX is installed neither here
nor on the GPU machine, and ``test_jax_bridge.py`` runs that part where it is."""
import sys
import types

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _standin():
    import torch
    jax = types.ModuleType("jax")

    class custom_vjp:
        def __init__(self, fun):
            self.fun, self.fwd, self.bwd = fun, None, None

        def defvjp(self, fwd, bwd):
            self.fwd, self.bwd = fwd, bwd

        def __call__(self, *args):
            return self.fun(*args)

    jax.custom_vjp = custom_vjp
    jax.dlpack = types.ModuleType("jax.dlpack")
    jax.dlpack.from_dlpack = lambda t: t
    jax.numpy = types.ModuleType("jax.numpy")
    jax.numpy.zeros_like = torch.zeros_like
    return jax


@pytest.fixture
def fake_jax(monkeypatch):
    jax = _standin()
    monkeypatch.setitem(sys.modules, "jax", jax)
    monkeypatch.setitem(sys.modules, "jax.dlpack", jax.dlpack)
    monkeypatch.setitem(sys.modules, "jax.numpy", jax.numpy)
    return jax


def test_bridge_vjp_matches_torch_autograd(fake_jax):
    import torch

    import updes_gb300 as U
    from updes_gb300.adjoint import pde_solver_torch
    from updes_gb300.jax_bridge import _TAPES, pde_solver_jax

    facets = {"South": "d", "West": "n", "North": "d", "East": "d"}
    cl = U.SquareCloud(Nx=10, Ny=9, facet_types=facets)
    X = cl.sorted_nodes
    k = 1.0 + 0.3 * np.sin(np.pi * X[:, 0])

    def op(x, center, rbf, monomial, fields):
        return fields[0] * U.nodal_laplacian(x, center, rbf, monomial) + U.nodal_value(x, center, rbf, monomial)

    rhs = lambda x, centers, rbf, fields: 1.0 + 0.0 * x[0]
    tmpl = {f: np.zeros(len(cl.facet_nodes[f])) for f in facets}
    rng = np.random.default_rng(0)
    cN = rng.standard_normal(len(cl.facet_nodes["North"]))
    cS = rng.standard_normal(len(cl.facet_nodes["South"]))
    dev = "cuda"
    f = pde_solver_jax(op, rhs, cl, U.polyharmonic, 1, tmpl, diff_operator_fields=True)
    bc = {"North": torch.tensor(cN, device=dev), "South": torch.tensor(cS, device=dev)}
    fields = (torch.tensor(k, device=dev),)

    vals, coeffs = f(bc, fields)  # the primal call
    (vals2, coeffs2), res = f.fwd(bc, fields)
    assert torch.equal(vals, vals2) and torch.equal(coeffs, coeffs2)
    assert len(_TAPES) == 1
    g_vals = 2.0 * vals2 / vals2.numel()  # d mean(vals^2) / d vals
    g_coeffs = torch.full_like(coeffs2, 0.25)  # and a loss term linear in the coefficients
    g_bc, g_fields = f.bwd(res, (g_vals, g_coeffs))
    assert len(_TAPES) == 0  # the tape is released by the backward pass

    tN = torch.tensor(cN, device=dev, requires_grad=True)
    tS = torch.tensor(cS, device=dev, requires_grad=True)
    tk = torch.tensor(k, device=dev, requires_grad=True)
    bcs = dict(tmpl)
    bcs.update(North=tN, South=tS)
    v, c = pde_solver_torch(op, rhs, cl, bcs, U.polyharmonic, 1, diff_args=[tk])
    loss = torch.mean(v ** 2) + 0.25 * torch.sum(c)
    loss.backward()
    for got, want in ((g_bc["North"], tN.grad), (g_bc["South"], tS.grad), (g_fields[0], tk.grad)):
        got, want = got.detach().cpu().numpy(), want.cpu().numpy()
        assert np.allclose(got, want, rtol=1e-10, atol=1e-13 * np.max(np.abs(want))), np.max(np.abs(got - want))


def test_bridge_without_differentiable_fields_returns_zero_field_gradients(fake_jax):
    import torch

    import updes_gb300 as U
    from updes_gb300.jax_bridge import pde_solver_jax

    facets = {"South": "d", "West": "d", "North": "d", "East": "d"}
    cl = U.SquareCloud(Nx=8, Ny=8, facet_types=facets)
    op = lambda x, center, rbf, monomial, fields: fields[0] * U.nodal_laplacian(x, center, rbf, monomial)
    rhs = lambda x, centers, rbf, fields: 0.0 * x[0]
    tmpl = {f: np.zeros(len(cl.facet_nodes[f])) for f in facets}
    f = pde_solver_jax(op, rhs, cl, U.polyharmonic, 1, tmpl)
    bc = {"North": torch.ones(len(cl.facet_nodes["North"]), dtype=torch.float64, device="cuda")}
    fields = (torch.full((cl.N,), 2.0, dtype=torch.float64, device="cuda"),)
    (vals, coeffs), res = f.fwd(bc, fields)
    g_bc, g_fields = f.bwd(res, (torch.ones_like(vals), torch.zeros_like(coeffs)))
    assert torch.count_nonzero(g_fields[0]) == 0
    assert torch.count_nonzero(g_bc["North"]) > 0
